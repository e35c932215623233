"""Build libdeeds_gpu.so and the deedsBCV / applyBCV / linearBCV command-line drivers in-tree.

    python -m deedsbcv_gb300.build          # or deedsbcv_gb300.build.build()

Everything is compiled for sm_103a only (GB300), with --fmad=false so that the
kernels keep the reference's separate IEEE multiply/add roundings, and host
code with -ffp-contract=off for the same reason.  Outputs go to
deedsbcv_gb300/_build/.  Translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libdeeds_gpu.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-Xptxas", "-v"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall", "-Wno-unused-function",
             f"-I{CUDA_HOME}/include"]

CU_SOURCES = ["mind.cu", "datacost.cu", "mst.cu", "stats.cu", "fusion.cu", "bp.cu", "transform.cu", "noalloc.cu", "soft.cu", "soft_warp.cu",
              "linear.cu"]
# soft.cu has no bit-exactness contract (its reference is a float64 definition),
# so it may contract multiply-adds and flush denormals (its operands never are:
# every square root and reciprocal square root argument is >= eps^2).
FMAD_SOURCES = {"soft.cu", "soft_warp.cu"}
CPP_SOURCES = ["pipeline.cpp", "tree_host.cpp", "linear_host.cpp", "gzio.cpp"]
CLI_SOURCES = {"deedsBCV": ["deedsBCV.cpp", "cli_common.cpp"], "applyBCV": ["applyBCV.cpp", "cli_common.cpp"],
               "applyBCVfloat": ["applyBCV.cpp", "cli_common.cpp"], "linearBCV": ["linearBCV.cpp", "cli_common.cpp"]}


def _run(cmd, log):
    p = subprocess.run(cmd, capture_output=True, text=True)
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + p.stdout + p.stderr)
    if p.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    return p


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, cli=True):
    """Compile everything; returns the library path.  Raises on any failure."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "deeds_gpu.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            flags = [("--fmad=true" if f == "--fmad=false" else f) for f in NVCC_FLAGS] + ["-ftz=true"] \
                if src in FMAD_SOURCES else NVCC_FLAGS
            jobs.append(([NVCC] + flags + ["-c", s, "-o", o], o + ".log"))
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append((["g++"] + CXX_FLAGS + ["-c", s, "-o", o], o + ".log"))
    with ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(lambda j: _run(*j), jobs))
    if force or jobs or not os.path.exists(LIB):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-lz"], LIB + ".log")
    if cli:
        build_cli(force=force)
    if verbose:
        print("built", LIB)
    return LIB


def build_cli(force=False):
    """The deedsBCV / applyBCV / applyBCVfloat / linearBCV executables (need zlib)."""
    lib_deps = [LIB]
    for exe, srcs in CLI_SOURCES.items():
        target = os.path.join(OUT, exe)
        paths = [os.path.join(CLI, s) for s in srcs]
        if not all(os.path.exists(p) for p in paths):
            continue
        deps = paths + lib_deps + [os.path.join(CLI, "cli_common.h"), os.path.join(ROOT, "include", "deeds_gpu.h")]
        if not force and not _stale(target, deps):
            continue
        defs = ["-DAPPLY_FLOAT=1"] if exe == "applyBCVfloat" else []
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{ROOT}/include"] + defs + paths +
             ["-o", target, f"-L{OUT}", "-ldeeds_gpu", "-lz", "-pthread", "-Wl,-rpath,$ORIGIN"], target + ".log")


def clean():
    shutil.rmtree(OUT, ignore_errors=True)


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
