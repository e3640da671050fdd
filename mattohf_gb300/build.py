"""Build the in-tree shared library ``mattohf_gb300/_lib/libmattohf.so``.

nvcc compiles each translation unit for sm_103a in parallel, then links one
shared object with the CUDA runtime linked statically (no torch types cross
the C ABI).  Run as ``python -m mattohf_gb300.build`` or via
``__graft_entry__.build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libmattohf.so")
DRIVER = os.path.join(OUT_DIR, "mattohf")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["ctx.cu", "k_hpsi.cu", "k_gs.cu", "k_table.cu", "noalloc.cu", "k_adjoint.cu", "k_spectra.cu", "k_fock_df.cu",
           "k_small.cu", "k_small_adj.cu"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _flags(verbose_ptxas: bool = False):
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--fmad=true",
         "-I" + CSRC, "-I" + os.path.join(HERE, "..", "include")] + ARCH
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int = 0) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "mattohf.h"))
    objs = []
    jobs_list = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or verbose_ptxas or not _newer(o, [s] + headers):
            jobs_list.append([nvcc(), "-c", s, "-o", o] + _flags(verbose_ptxas))
    n = jobs or min(len(jobs_list), os.cpu_count() or 4) or 1
    errors = []
    with cf.ThreadPoolExecutor(max_workers=n) as ex:
        for cmd, res in zip(jobs_list, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs_list)):
            if verbose_ptxas and res.stderr:
                sys.stderr.write(res.stderr)
            if res.returncode != 0:
                errors.append(" ".join(cmd) + "\n" + res.stdout + res.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    relinked = False
    if force or jobs_list or not os.path.exists(LIB):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n" + res.stdout + res.stderr)
        relinked = True
    build_driver(force or relinked)
    return LIB


def build_driver(force: bool = False) -> str:
    """The C++ drop-in driver ``_lib/mattohf`` (reads input.dat, writes the reference's outputs)."""
    src = os.path.join(CSRC, "mattohf_main.cpp")
    hdr = os.path.join(HERE, "..", "include", "mattohf.h")
    if force or not _newer(DRIVER, [src, hdr, LIB]):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I" + os.path.join(HERE, "..", "include"), src, "-o", DRIVER,
               "-L" + OUT_DIR, "-lmattohf", "-Wl,-rpath,$ORIGIN"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("driver build failed:\n" + res.stdout + res.stderr)
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
