"""In-tree build of libthmm_gb300.so (sm_103a) with nvcc.

Each translation unit is compiled in parallel into parallel_tree_hmm_gb300/_build
and linked into parallel_tree_hmm_gb300/libthmm_gb300.so. Only nvcc and the host
C++ compiler are needed (no cmake, no torch extension machinery).
"""
from __future__ import annotations

import concurrent.futures
import os
import pathlib
import shutil
import subprocess

PACKAGE = pathlib.Path(__file__).resolve().parent
ROOT = PACKAGE.parent
CSRC = PACKAGE / "csrc"
BUILD = PACKAGE / "_build"
LIBRARY = PACKAGE / "libthmm_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = [
    "-std=c++20",
    "-O3",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-ffp-contract=off",
    f"-I{ROOT / 'include'}",
    f"-I{CSRC}",
]
SOURCES = [
    # Slowest first: the build compiles them in parallel.
    "engine_linear_fd_rev_large.cu",
    "engine_linear_dd_rev_large.cu",
    "engine_linear_ff_rev_large.cu",
    "engine_linear_df_rev_large.cu",
    "engine_linear_fd_fwd_large.cu",
    "engine_linear_dd_fwd_large.cu",
    "engine_linear_ff_fwd_large.cu",
    "engine_linear_df_fwd_large.cu",
    "engine_linear_fd_rev_small.cu",
    "engine_linear_dd_rev_small.cu",
    "engine_linear_ff_rev_small.cu",
    "engine_linear_df_rev_small.cu",
    "engine_linear_fd_fwd_small.cu",
    "engine_linear_dd_fwd_small.cu",
    "engine_linear_ff_fwd_small.cu",
    "engine_linear_df_fwd_small.cu",
    "engine_maximum_f64.cu",
    "engine_maximum_f32.cu",
    "engine_sample_f64.cu",
    "engine_sample_f32.cu",
    "engine_wide.cu",
    "engine_phase.cu",
    "engine_wide_phase.cu",
    "engine_phase_groups_32_f64.cu",
    "engine_phase_groups_32_f32.cu",
    "engine_phase_groups_28_f32.cu",
    "engine_phase_groups_24_f32.cu",
    "engine_phase_groups_20_f32.cu",
    "engine_phase_groups_16_f64.cu",
    "engine_phase_groups_16_f32.cu",
    "engine_phase_groups_8_f64.cu",
    "engine_phase_groups_8_f32.cu",
    "engine_linear_f32.cu",
    "engine_linear_f64.cu",
    "engine_maximum.cu",
    "engine_sample.cu",
    "static_scratch.cu",
    "runtime.cc",
    "program.cc",
    "phase.cc",
    "btrc_plan.cc",
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required")
    return path


def _compile(source: str) -> pathlib.Path:
    src = CSRC / source
    obj = BUILD / (source + ".o")
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(
        (ROOT / "include").rglob("*.h"))
    newest = max([src.stat().st_mtime] + [h.stat().st_mtime for h in headers])
    if obj.exists() and obj.stat().st_mtime >= newest:
        return obj
    cmd = [nvcc(), *COMMON, *ARCH, "-c", str(src), "-o", str(obj)]
    if source.endswith(".cu"):
        cmd[1:1] = ["-x", "cu"]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"nvcc failed for {source}:\n{result.stdout}\n{result.stderr}")
    return obj


def build_library(jobs: int | None = None) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as pool:
        objects = list(pool.map(_compile, SOURCES))
    if LIBRARY.exists() and LIBRARY.stat().st_mtime >= max(o.stat().st_mtime for o in objects):
        return LIBRARY
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objects)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"link failed:\n{result.stdout}\n{result.stderr}")
    os.replace(tmp, LIBRARY)
    return LIBRARY


def build_cpp_tests() -> list[pathlib.Path]:
    """Compiles tests/cpp/accelerator_dropin_test.cc (C++ API drop-in check)
    in the FP64 and FP32 precisions against the in-tree library and the
    oracle; the GPU tests run the binaries."""
    source = ROOT / "tests" / "cpp" / "accelerator_dropin_test.cc"
    outputs = []
    for tag, defines in (("f64", []), ("f32", ["-DTREE_HMM_USE_FLOAT=1"])):
        binary = source.with_name(f"accelerator_dropin_test_{tag}")
        inputs = [source, LIBRARY, ROOT / "oracle" / "liboracle.so",
                  *(ROOT / "include").rglob("*.h")]
        if binary.exists() and binary.stat().st_mtime >= max(p.stat().st_mtime for p in inputs):
            outputs.append(binary)
            continue
        cuda_include = pathlib.Path(nvcc()).resolve().parent.parent / "include"
        cmd = [os.environ.get("CXX", "g++"), "-std=c++20", "-O2", *defines,
               f"-I{ROOT / 'include'}", f"-I{ROOT / 'oracle'}", f"-I{cuda_include}",
               str(source), "-o", str(binary), f"-L{PACKAGE}", "-lthmm_gb300",
               f"-L{ROOT / 'oracle'}", "-loracle", f"-Wl,-rpath,{PACKAGE}",
               f"-Wl,-rpath,{ROOT / 'oracle'}"]
        result = subprocess.run(cmd, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError(f"C++ test build failed:\n{result.stderr}")
        outputs.append(binary)
    return outputs


def build_oracle(reference: bool = True) -> None:
    """Builds the C oracle (test infrastructure) and, when the reference tree
    is present, the reference CPU library and tests under oracle/_ref."""
    oracle_dir = ROOT / "oracle"
    subprocess.run(["make", "-s", "-C", str(oracle_dir)], check=True)
    # The reference checkout: $THMM_REFERENCE, else `reference` beside the repo.
    ref = os.environ.get("THMM_REFERENCE", str(ROOT.parent / "reference"))
    if reference and os.path.isdir(os.path.join(ref, "src")):
        subprocess.run(["make", "-s", "-C", str(oracle_dir), "ref", f"REF={ref}"], check=True)
        # Copies of the reference's accelerator suite for machines without
        # the reference tree (built there by tests/test_gpu_ref_suite.py).
        subprocess.run(["make", "-s", "-C", str(oracle_dir), "ref-suite-stage", f"REF={ref}"],
                       check=True)


if __name__ == "__main__":
    print(build_library())
    build_oracle()
    print(build_cpp_tests())
