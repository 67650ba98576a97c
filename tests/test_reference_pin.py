"""Pins the oracle to the reference itself, where the reference tree is
available (this needs oracle/_ref, built by `make -C oracle ref`).

* The reference's own CPU tests, compiled unmodified against this project's
  restated planner, pass (FP64 and FP32 builds).
* The oracle and the reference library agree bit for bit on random trees,
  states and factors with exact zeros, for every operation and every error.
"""
import pathlib
import subprocess

import numpy as np
import pytest

from oracle import bridge
from parallel_tree_hmm_gb300 import synthetic

REF = pathlib.Path(__file__).resolve().parents[1] / "oracle" / "_ref"
needs_reference = pytest.mark.skipif(
    not bridge.Reference.available(np.float64) or not bridge.Reference.available(np.float32),
    reason="reference build (oracle/_ref) not present")


@needs_reference
@pytest.mark.parametrize("binary", [
    "inference_test_f64", "inference_test_f32", "gpu_device_algebra_test_f64",
    "gpu_device_algebra_test_f32", "accelerator_path_storage_test"])
def test_reference_cpu_tests_pass_against_planner(binary):
    path = REF / binary
    if not path.exists():
        pytest.skip(f"{binary} not built")
    result = subprocess.run([str(path)], capture_output=True, text=True, timeout=300)
    assert result.returncode == 0, result.stderr


def _outcome(call):
    try:
        return ("ok", call())
    except bridge.OracleError as error:
        return ("error", error.status)


def _equal(a, b):
    if a[0] != b[0]:
        return False
    if a[0] == "error":
        return a[1] == b[1]
    x, y = a[1], b[1]
    if isinstance(x, tuple):
        return all(np.array_equal(np.asarray(p), np.asarray(q), equal_nan=True)
                   for p, q in zip(x, y))
    return np.array_equal(np.asarray(x), np.asarray(y), equal_nan=True)


@needs_reference
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_oracle_matches_reference_bit_for_bit(dtype, thmm):
    rng = np.random.default_rng(99 if dtype == np.float64 else 98)
    reference = bridge.Reference(dtype)
    for _ in range(60):
        n = int(rng.integers(1, 90))
        states = int(rng.integers(1, 7))
        parents = synthetic.random_recursive(rng, n)
        plan = thmm.Plan(parents)
        nodes = (rng.random(n * states) * 0.9 + 0.1).astype(dtype)
        edges = (rng.random((n - 1) * states * states) * 0.9 + 0.1).astype(dtype)
        nodes[rng.random(nodes.size) < 0.03] = 0
        edges[rng.random(edges.size) < 0.03] = 0
        uniforms = rng.random(n).astype(dtype)
        handle = reference.model(parents, states)
        try:
            pairs = [
                (lambda: reference.log_partition(handle, nodes, edges),
                 lambda: bridge.log_partition(plan, states, nodes, edges, dtype)),
                (lambda: reference.partition(handle, nodes, edges),
                 lambda: bridge.partition(plan, states, nodes, edges, dtype)),
                (lambda: reference.marginals(handle, nodes, edges, n, n - 1, states),
                 lambda: bridge.marginals(plan, states, nodes, edges, dtype)),
                (lambda: reference.maximum(handle, nodes, edges, n),
                 lambda: bridge.maximum(plan, states, nodes, edges, dtype)),
                (lambda: reference.sample(handle, nodes, edges, uniforms, n),
                 lambda: bridge.sample(plan, states, nodes, edges, uniforms, dtype)),
            ]
            for ref_call, oracle_call in pairs:
                assert _equal(_outcome(ref_call), _outcome(oracle_call))
        finally:
            reference.destroy(handle)
