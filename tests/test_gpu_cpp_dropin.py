"""Runs the C++ drop-in check (tests/cpp/accelerator_dropin_test.cc): code
written against the reference's tree_hmm::cuda API, compiled against this
library's headers, in the FP64 and FP32 builds of tree_hmm::Scalar."""
import pathlib
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = pathlib.Path(__file__).resolve().parent


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_cpp_accelerator_api_drop_in(gpu, tag):
    binary = HERE / "cpp" / f"accelerator_dropin_test_{tag}"
    if not binary.exists():
        from parallel_tree_hmm_gb300 import build

        build.build_cpp_tests()
    result = subprocess.run([str(binary)], capture_output=True, text=True, timeout=600)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "checks passed" in result.stdout
