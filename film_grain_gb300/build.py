"""Build the film_grain_gb300 shared library in-tree (film_grain_gb300/_build/libfg_gb300.so).

sm_103a only: every CUDA translation unit is compiled with
``-gencode arch=compute_103a,code=sm_103a``.  The coverage path needs IEEE f32/f64 rounding in
Rust's (unfused) expression order, so the integrator units use ``--fmad=false`` (no FMA
contraction), keep IEEE division and square root, and the host code is compiled with
``-ffp-contract=off``.  The CUDA runtime is linked statically so the library is self-contained
next to any other runtime in the process.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfg_gb300.so")
ROOT = os.path.dirname(HERE)

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_EXACT = ["fg_pixelwise.cu", "fg_grainwise.cu", "fg_capi.cu", "fg_noalloc.cu", "fg_batch.cu", "fg_lambda.cu"]
CU_FAST = ["fg_surrogate.cu", "fg_sg_tc.cu"]
CPP = ["fg_host.cpp"]

NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
               "-I", os.path.join(ROOT, "include"), "-I", CSRC, *ARCH]


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".cpp"))]


def _needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = _sources() + [os.path.join(ROOT, "include", "film_grain_gb300.h"), os.path.abspath(__file__)]
    return any(os.path.getmtime(s) > t for s in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA and host unit for sm_103a and link libfg_gb300.so; returns its path."""
    if not force and not _needs_build():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for f in CU_EXACT:
        obj = os.path.join(OUT, f + ".o")
        jobs.append(([NVCC, *NVCC_COMMON, "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
                      "-Xptxas", "-v", "-c", os.path.join(CSRC, f), "-o", obj], obj))
    for f in CU_FAST:
        obj = os.path.join(OUT, f + ".o")
        jobs.append(([NVCC, *NVCC_COMMON, "-Xptxas", "-v", "-c", os.path.join(CSRC, f), "-o", obj], obj))
    for f in CPP:
        obj = os.path.join(OUT, f + ".o")
        jobs.append((["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fvisibility=hidden",
                      "-pthread", "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", "/usr/local/cuda/include",
                      "-c", os.path.join(CSRC, f), "-o", obj], obj))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for log in logs:
            sys.stderr.write(log)
    with open(os.path.join(OUT, "ptxas.log"), "w") as fh:
        fh.write("\n".join(logs))
    tmp = LIB + ".tmp"
    _run([NVCC, "-shared", *ARCH, "-cudart", "static", "-o", tmp, *[j[1] for j in jobs],
          "-Xcompiler", "-pthread", "-lpthread", "-lrt", "-ldl"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
