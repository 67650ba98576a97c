"""The reference's own accelerator suite, unmodified, against this library.

tests/cuda_test.cc of the reference, with its accelerator_test.h and
gpu_backend_test.inc, is the contract the reference's CUDA backend is tested
against: batch 257, staged inputs, a 4096-node chain, K = 9, a 17-leaf star,
categorical log Z bit-equal to dense, MAP states and posterior samples equal
to the CPU library, residency rules and their exceptions, marginals with
exact zeros. `make -C oracle ref-suite` builds it from staged copies of the
reference files (oracle/_ref/suite, made by `make -C oracle ref-suite-stage`
where the reference tree is present; never committed) against
tests/cpp/ref_suite/tree_hmm/cuda.h, which forwards "tree_hmm/cuda.h" to this
library's tree_hmm::gb300, and the reference's own src/inference.cc for the
suite's CPU comparisons. Both precisions of the suite must exit 0.
"""
import pathlib
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = pathlib.Path(__file__).resolve().parents[1]
SUITE = ROOT / "oracle" / "_ref" / "suite"


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_reference_accelerator_suite_passes(gpu, precision):
    if not (SUITE / "tests" / "cuda_test.cc").exists():
        pytest.skip("reference suite not staged (make -C oracle ref-suite-stage)")
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref-suite"], check=True)
    binary = ROOT / "oracle" / "_ref" / f"ref_suite_{precision}"
    result = subprocess.run([str(binary)], capture_output=True, text=True, timeout=600)
    assert result.returncode == 0, result.stdout[-4000:] + result.stderr[-4000:]
