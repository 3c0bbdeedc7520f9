"""Builds libsimgb.so in-tree with nvcc for sm_103a (no CMake, no torch extension).

    python -m simbuca_gb300.build

Translation units are compiled in parallel into simbuca_gb300/_build/ and linked
into simbuca_gb300/libsimgb.so (CUDA runtime linked statically).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
OUT = os.path.join(PKG, "libsimgb.so")
UNITS = ["coulomb.cu", "dp45.cu", "capi.cu", "aux_kernels.cu", "noalloc.cu", "check.cu", "fused.cu",
         "proposer.cu", "cloud_io.cu", "observe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libsimgb needs the CUDA toolkit to build")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, "sg_internal.cuh"), os.path.join(CSRC, "fp32c_math.cuh"),
               os.path.join(CSRC, "dp_tableau.cuh"),
               os.path.join(os.path.dirname(PKG), "include", "simgb.h")]
    procs, objs = [], []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc()] + ARCH + FLAGS + ["-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((u, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                              stderr=subprocess.STDOUT, text=True)))
    failed = []
    for u, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((u, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n".join(f"--- {u}\n{o}" for u, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    if force or _stale(OUT, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", OUT] + objs + ["-lcudart_static", "-lrt",
                                                                 "-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(OUT)
