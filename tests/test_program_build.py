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


def test_phase_schedule_records_and_host_run(tmp_path):
    """The level-synchronous phase schedule (csrc/phase.h): record indices in
    bounds, every path produced before use and consumed once, and a double
    precision host run of the records, whole and striped, equal to the
    oracle's log Z and marginals (tests/cpp/phase_plan_test.cc)."""
    cxx, cc = shutil.which("g++"), shutil.which("gcc")
    include = cuda_include()
    if cxx is None or cc is None or include is None:
        pytest.skip("needs g++, gcc and the CUDA headers")
    oracle_object = tmp_path / "oracle.o"
    subprocess.run([cc, "-std=c11", "-O2", "-ffp-contract=off", "-c",
                    str(ROOT / "oracle" / "oracle.c"), "-o", str(oracle_object)], check=True)
    binary = tmp_path / "phase_plan_test"
    subprocess.run([cxx, "-std=c++20", "-O2", "-pthread", f"-I{ROOT / 'include'}",
                    f"-I{CSRC}", f"-I{ROOT / 'oracle'}", f"-I{include}",
                    str(ROOT / "tests" / "cpp" / "phase_plan_test.cc"),
                    str(CSRC / "program.cc"), str(CSRC / "phase.cc"),
                    str(CSRC / "btrc_plan.cc"), str(oracle_object), "-lm", "-o", str(binary)],
                   check=True)
    result = subprocess.run([str(binary)], capture_output=True, text=True, timeout=600)
    assert result.returncode == 0, result.stdout + result.stderr
    assert "passed" in result.stdout
