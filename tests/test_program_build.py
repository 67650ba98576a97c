"""Parallel compilation of tree programs gives exactly the one-thread arrays
(tests/cpp/program_build_test.cc, compiled with the host compiler; no GPU)."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "parallel_tree_hmm_gb300" / "csrc"


def cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    path = pathlib.Path(nvcc).resolve().parent.parent / "include"
    return path if (path / "cuda_runtime.h").exists() else None


def test_parallel_program_build_matches_serial(tmp_path):
    cxx = shutil.which("g++")
    include = cuda_include()
    if cxx is None or include is None:
        pytest.skip("needs g++ and the CUDA headers")
    binary = tmp_path / "program_build_test"
    subprocess.run([cxx, "-std=c++20", "-O2", "-pthread", f"-I{ROOT / 'include'}",
                    f"-I{CSRC}", f"-I{include}", str(ROOT / "tests" / "cpp" /
                                                     "program_build_test.cc"),
                    str(CSRC / "program.cc"), str(CSRC / "btrc_plan.cc"), "-o", str(binary)],
                   check=True)
    result = subprocess.run([str(binary)], capture_output=True, text=True, timeout=300)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "passed" in result.stdout
