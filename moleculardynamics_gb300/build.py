"""Builds the engine in-tree: libmdgb.so (CUDA sm_103a + host C++) and mdgb_run.

nvcc compiles each translation unit in parallel with
``-gencode arch=compute_103a,code=sm_103a``; nothing is pip-installed.  The
library exports the C ABI of include/mdgb.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libmdgb.so")
RUN = os.path.join(PKG, "mdgb_run")

CU_SOURCES = ["md_neighbor.cu", "md_forces.cu", "md_cluster.cu", "md_surrogate.cu", "md_integrate.cu", "md_output.cu", "md_engine.cu",
              "md_refshim.cu", "md_static.cu", "md_diag.cu"]
CPP_SOURCES = ["md_io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC",
                  "-diag-suppress", "1444", "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmdgb.so")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(ROOT, "include", "mdgb.h")]


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libmdgb.so and mdgb_run if any source changed; returns the .so path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    jobs = []
    for src in CU_SOURCES + CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        if force or _stale(o, [s] + headers):
            lang = ["-x", "cu"] if src.endswith(".cu") else []
            jobs.append([nvcc] + NVFLAGS + lang + ["-c", s, "-o", o])
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, s + ".o") for s in CU_SOURCES + CPP_SOURCES]
    if force or jobs or _stale(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"])
        os.replace(LIB + ".tmp", LIB)
    drv = os.path.join(CSRC, "mdgb_run.cpp")
    if force or _stale(RUN, [drv, LIB] + headers):
        run([nvcc] + ARCH + ["-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-x", "cu",
                             drv, "-o", RUN + ".tmp", "-L", PKG, "-lmdgb",
                             "-Xlinker", "-rpath=$ORIGIN"])
        os.replace(RUN + ".tmp", RUN)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
