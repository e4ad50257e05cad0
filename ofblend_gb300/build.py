"""Builds libflof_gb300.so, the CUDA library behind the C ABI of
include/flof_gb300.h, for sm_103a only.

Each translation unit is compiled in parallel with -fmad=false (multiplies
and adds rounded separately, as in the reference's x86 build) and linked into
one shared library next to this file.  Run as `python -m ofblend_gb300.build`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflof_gb300.so")
SOURCES = ["flof_ops.cu", "flof_solve.cu", "flof_stencil.cu", "flof_tma.cu", "flof_cond.cu",
           "flof_host.cu", "flof_ext.cu", "flof_uni.cu", "flof_batch.cu", "flof_mixed.cu",
           "flof_net.cu", "flof_conv_tc.cu", "flof_model.cu", "flof_noalloc.cu",
           "flof_strict.cu", "flof_mg.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build flof-gb300")


def flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
        "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
        # host-side parameter arithmetic (grid factors, slice times) must not
        # be contracted to FMA either: GCC does so by default on aarch64
        "-Xcompiler", "-ffp-contract=off",
        "-Xptxas", "-warn-spills",
        "-I", CSRC, "-I", os.path.join(os.path.dirname(HERE), "include"),
    ]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "flof_gb300.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc] + flags() + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fPIC", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
