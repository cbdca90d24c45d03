"""In-tree build of liboofem_gb300.so (sm_103a) with nvcc; no CMake.

Each CUDA translation unit is compiled in parallel to an object file under
oofem_gb300/_build/, then linked into oofem_gb300/liboofem_gb300.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liboofem_gb300.so")
SOURCES = ["capi.cu", "scan.cu", "pattern.cu", "element.cu", "assembly.cu", "solver.cu", "newton.cu", "batch.cu", "halfsell.cu", "deckparse.cu", "icprec.cu", "direct.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, "internal.cuh"), os.path.join(CSRC, "reduce.cuh"), os.path.join(CSRC, "tcgen05.cuh"),
               os.path.join(os.path.dirname(HERE), "include", "oofem_gb300.h")]
    cc = nvcc()
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + headers):
            jobs.append([cc, *ARCH, *FLAGS, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode != 0:
                    print(" ".join(j))
                    print(r.stdout, r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed for {j[-3]}")
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        r = subprocess.run([cc, *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"], capture_output=True, text=True)
        if r.returncode != 0:
            print(r.stdout, r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
