"""Builds libqssgpu.so (the GB300 implementation of the lsmpqs C API) in-tree.

    python lsmpqs-1.0_gb300/build.py [--jobs N] [--verbose]

Every CUDA translation unit is compiled for sm_103a only, with --fmad=false:
the kernels restate the reference's FP64 arithmetic operation by operation,
and a fused multiply-add would round differently.  Host code is compiled
without floating-point contraction for the same reason.  The exception is
the adjoint's reverse kernels (qss_adjoint.cu): a gradient has no reference
bit pattern to match, so they may fuse multiply-adds (fewer FP64
instructions on the pipe that bounds them); the forward model they
differentiate runs in the other, uncontracted translation units.  Translation units
are compiled in parallel; the shared library links the CUDA runtime
statically so it only needs the driver at run time.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libqssgpu.so")
OBJ = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-fast-math",
    "-Xptxas", "-warn-spills",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


# translation units allowed to contract a * b + c into one FMA
FMAD_UNITS = {"qss_adjoint.cu"}


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    flags = NVCC_FLAGS
    if os.path.basename(src) in FMAD_UNITS:
        flags = ["--fmad=true" if f == "--fmad=false" else f for f in NVCC_FLAGS]
    cmd = [nvcc()] + flags + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-fast-math", "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return obj


def build(jobs: int = 0, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    cmd = [nvcc()] + ARCH + ["-shared", "-o", OUT] + objs + ["-lpthread", "-ldl", "-lrt"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=0)
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.jobs, a.verbose))
    sys.exit(0)
