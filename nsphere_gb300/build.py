"""In-tree build of libnsg.so (sm_103a only).

Each ``csrc/*.cu`` file compiles in parallel to an object under ``_build/`` and
the objects link into ``nsphere_gb300/libnsg.so``.  Integrator arithmetic uses
explicit round-to-nearest intrinsics, so the result does not depend on
``--fmad``; the flag is still off for the integrator file as a second guard.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnsg.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]
NO_FMAD = {"nsg_integrate.cu", "nsg_mlp.cu", "nsg_ics.cu", "nsg_post.cu", "nsg_track.cu", "nsg_density.cu"}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libnsg needs the CUDA 13 toolkit")


def _needs(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")))
    objs, jobs = [], []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _needs(obj, [src, *headers]):
            flags = list(NVCC_FLAGS)
            if os.path.basename(src) in NO_FMAD:
                flags += ["--fmad=false", "-Xcompiler=-ffp-contract=off"]
            jobs.append([nvcc, *ARCH, *flags, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or r.returncode != 0:
                    print(" ".join(cmd))
                    print(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed on " + cmd[-3])
    if force or jobs or _needs(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        if verbose:
            print("linked", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
