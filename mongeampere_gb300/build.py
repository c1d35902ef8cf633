"""Build ``libma_gb300.so`` (the C-ABI library) for sm_103a with nvcc.

Each ``csrc/*.cu`` translation unit is compiled in parallel, then linked into a
shared library next to this file, in ``_build/``.  No CMake, no torch extension
machinery: the library exposes a plain C ABI (``include/ma.h``).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libma_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I", SRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    os.makedirs(OUT, exist_ok=True)
    cus = sorted(glob.glob(os.path.join(SRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(SRC, "*.cuh")) + glob.glob(os.path.join(SRC, "*.h")) +
                     glob.glob(os.path.join(ROOT, "include", "*.h")))
    objs = []
    jobs = []
    nv = nvcc()
    for cu in cus:
        obj = os.path.join(OUT, os.path.basename(cu)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [cu] + headers):
            cmd = [nv, *ARCH, *NVFLAGS, *(extra or []), "-c", cu, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, cmd, capture_output=True, text=True) for cmd in jobs]
            for cmd, fu in zip(jobs, futs):
                r = fu.result()
                if verbose or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
