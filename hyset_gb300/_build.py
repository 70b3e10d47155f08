"""Build recipe for the native parts, in-tree (no pip install).

    python -m hyset_gb300._build            # everything
Products (git-ignored):
    hyset_gb300/libhyset_gb300.so   CUDA kernels + C ABI (sm_103a only)
    hyset_gb300/libhyset_synth.so   seeded synthetic collections (host C++)
    oracle/liboracle.so             CPU checker (test infrastructure)
    oracle/_ref/ref_join            the reference's own host join (only where its sources exist)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhyset_gb300.so")
SYNTH = os.path.join(PKG, "libhyset_synth.so")

CUDA_SOURCES = ["primitives.cu", "join.cu", "join_tm.cu", "batch.cu", "mlp.cu", "stats.cu", "parse.cu", "noalloc.cu",
                # host side of the C ABI
                "capi.cu", "collection.cu", "bounds.cu", "index_host.cu", "plan.cu", "join_host.cu", "pipeline.cu",
                "batch_host.cu", "handlers.cu", "verifier.cu", "ring.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    # the bound tables are computed on the host with the reference's double
    # expressions; no multiply-add contraction may change them
    "-Xcompiler", "-fPIC,-ffp-contract=off",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_cuda(force: bool = False, verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "hyset_gb300.h"))
    jobs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose else []) + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(CUDA_SOURCES)) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                sys.stderr.write(r.stderr)
    objs = [os.path.join(BUILD, s + ".o") for s in CUDA_SOURCES]
    if force or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs)
    return LIB


def build_synth(force: bool = False) -> str:
    src = os.path.join(CSRC, "synth.cpp")
    hdr = os.path.join(ROOT, "include", "hyset_gb300_synth.h")
    if force or _stale(SYNTH, [src, hdr]):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-o", SYNTH, src])
    return SYNTH


def build_oracle(force: bool = False) -> None:
    odir = os.path.join(ROOT, "oracle")
    _run(["make", "-C", odir] + (["-B"] if force else []) + ["liboracle.so"])
    # the reference's own host join, where its source tree exists (the recipe
    # in oracle/Makefile knows where it lies; HYSET_REFERENCE_ROOT overrides)
    ref = os.environ.get("HYSET_REFERENCE_ROOT")
    _run(["make", "-C", odir] + ([f"REFROOT={ref}"] if ref else []) + ["ref-if-present"])


def build_all(force: bool = False, verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_cuda, force, verbose), ex.submit(build_synth, force), ex.submit(build_oracle, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print("built", LIB)
