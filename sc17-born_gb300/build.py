"""Builds libborn_gb300.so (the CUDA kernels and the C ABI) for sm_103a.

Each translation unit is compiled in parallel with nvcc, then linked into
``_build/libborn_gb300.so`` next to this file (in-tree, git-ignored).  Usage:
``python sc17-born_gb300/build.py [--force] [-v]``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libborn_gb300.so")

SOURCES = ["born_step.cu", "born_step_bf16.cu", "born_step_f16.cu",
           "born_step_f32fused.cu", "born_step_f32exact.cu",
           "born_api.cu", "born_operator.cu", "born_batch.cu",
           "born_noalloc.cu", "born_velocity.cu", "born_stream.cu",
           "born_host.cc",
           "born_sepio.cc"]
HEADERS = ["born_step.cuh", "born_step_impl.cuh", "born_host.h",
           "born_internal.h", "born_couple.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required")


def _flags(src: str, verbose: bool) -> list[str]:
    f = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
         "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if src.endswith(".cu"):
        f = ARCH + ["-lineinfo"] + f
        if verbose:
            f += ["-Xptxas", "-v"]
    else:
        f = ["-x", "c++"] + f
    return f


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(ROOT, "include", "born_gb300.h")]
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, __file__] + hdrs):
            jobs.append([nvcc, "-c", src, "-o", obj] + _flags(s, verbose))
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd, res in zip(jobs, ex.map(
                lambda c: subprocess.run(c, capture_output=True, text=True),
                jobs)):
            if res.returncode != 0 or verbose:
                sys.stderr.write(res.stdout + res.stderr)
            if res.returncode != 0:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, "-shared", "-o", LIB] + ARCH + objs
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError("link failed: " + " ".join(cmd))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
