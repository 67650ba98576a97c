"""The oracle (C restatement of src/inference.cc) against the golden fixtures
produced by the reference's own build (tests/golden/make_golden.py).

On x86-64 the oracle reproduces the reference bit for bit, in FP64 and FP32,
for log Z, Z, marginals, MAP and posterior samples, including the cases where
the reference reports a domain error. Elsewhere the C library's exp/log may
round differently in the last bit, so values are compared within 8 ulps and
discrete outputs exactly.
"""
import pathlib
import platform

import numpy as np
import pytest

from oracle import bridge

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "reference_cpu.npz"
EXACT = platform.machine() in ("x86_64", "AMD64")


def _cases():
    data = np.load(GOLDEN)
    names = sorted({key.split("/")[0] for key in data.files})
    return data, names


DATA, NAMES = _cases()


def _same(actual, expected, dtype):
    actual = np.asarray(actual, dtype=dtype)
    expected = np.asarray(expected, dtype=dtype)
    if EXACT:
        return np.array_equal(actual, expected, equal_nan=True)
    eps = np.finfo(dtype).eps
    return np.allclose(actual, expected, rtol=8 * eps, atol=8 * eps, equal_nan=True)


@pytest.mark.parametrize("tag,dtype", [("f64", np.float64), ("f32", np.float32)])
@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_reference(name, tag, dtype, thmm):
    parents = DATA[f"{name}/parents"]
    states = int(DATA[f"{name}/states"])
    plan = thmm.Plan(parents)
    nodes = DATA[f"{name}/{tag}/nodes"]
    edges = DATA[f"{name}/{tag}/edges"]
    uniforms = DATA[f"{name}/{tag}/uniforms"]
    key = f"{name}/{tag}/"
    assert _same(bridge.log_partition(plan, states, nodes, edges, dtype),
                 DATA[key + "log_partition"], dtype)
    assert _same(bridge.partition(plan, states, nodes, edges, dtype),
                 DATA[key + "partition"], dtype)
    if key + "marginal_status" in DATA.files:
        with pytest.raises(bridge.OracleError) as error:
            bridge.marginals(plan, states, nodes, edges, dtype)
        assert error.value.status == int(DATA[key + "marginal_status"])
    else:
        log_z, z, node_m, edge_m = bridge.marginals(plan, states, nodes, edges, dtype)
        assert _same(log_z, DATA[key + "marginal_log_partition"], dtype)
        assert _same(node_m, DATA[key + "node_marginals"], dtype)
        assert _same(edge_m, DATA[key + "edge_marginals"], dtype)
    if key + "map_status" in DATA.files:
        with pytest.raises(bridge.OracleError):
            bridge.maximum(plan, states, nodes, edges, dtype)
    else:
        weight, states_map = bridge.maximum(plan, states, nodes, edges, dtype)
        assert _same(weight, DATA[key + "map_log_weight"], dtype)
        assert np.array_equal(states_map, DATA[key + "map_states"])
    if key + "sample_status" in DATA.files:
        with pytest.raises(bridge.OracleError):
            bridge.sample(plan, states, nodes, edges, uniforms, dtype)
    else:
        sample = bridge.sample(plan, states, nodes, edges, uniforms, dtype)
        if EXACT:
            assert np.array_equal(sample, DATA[key + "sample_states"])


def test_chain_known_answers(thmm):
    # A unary chain with node factor 1/2 everywhere: log Z = n log(1/2) and
    # every marginal is 1; with two states and a fixed transition the root
    # factor is absorbed: log Z = (n - 1) log(1/2).
    n = 4096
    plan = thmm.Plan(np.arange(-1, n - 1))
    log_z = bridge.log_partition(plan, 1, np.full(n, 0.5), np.ones(n - 1))
    assert abs(log_z - n * np.log(0.5)) <= 1e-10 * n
    log_z, z, node_m, edge_m = bridge.marginals(plan, 1, np.full(n, 0.5), np.ones(n - 1))
    assert z == 0.0 and abs(log_z - n * np.log(0.5)) <= 1e-10 * n
    assert np.allclose(node_m, 1.0) and np.allclose(edge_m, 1.0)
    edges = np.tile([0.9, 0.1, 0.2, 0.8], n - 1)
    log_z, _, node_m, edge_m = bridge.marginals(plan, 2, np.full(2 * n, 0.5), edges)
    assert abs(log_z - (n - 1) * np.log(0.5)) <= 1e-9 * n
    assert np.allclose(node_m.reshape(n, 2).sum(1), 1.0)
    assert np.allclose(edge_m.reshape(n - 1, 4).sum(1), 1.0)


def test_oracle_rejects_invalid_factors(thmm):
    plan = thmm.Plan([-1, 0])
    for bad in (-1.0, np.inf, np.nan):
        with pytest.raises(bridge.OracleError) as error:
            bridge.marginals(plan, 2, np.array([1, bad, 1, 1]), np.ones(4))
        assert error.value.status == bridge.ORACLE_INVALID_ARGUMENT
    with pytest.raises(bridge.OracleError):
        bridge.sample(plan, 2, np.ones(4), np.ones(4), np.array([0.5, 1.0]))
