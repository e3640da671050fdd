"""Compile the oracle's C restatement (``oracle/cref``) into ``oracle/_build/libmattohf_cref.so``.

Test infrastructure: used by the test-suite and by bench.py's CPU-baseline
legs only.  Plain gcc + OpenMP, portable flags (builds on x86-64 and aarch64).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cref", "mattohf_cref.c")
OUT = os.path.join(HERE, "_build", "libmattohf_cref.so")


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    cc = shutil.which("gcc") or "cc"
    cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", SRC, "-o", OUT, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("cref build failed:\n" + res.stderr)
    return OUT


def load():
    lib = C.CDLL(build())
    D = C.POINTER(C.c_double)
    P = C.c_void_p
    lib.cref_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, D, D, D]
    lib.cref_create.restype = P
    lib.cref_destroy.argtypes = [P]
    lib.cref_hpsi.argtypes = [P, D, D, C.c_int, C.c_double, D]
    lib.cref_observables.argtypes = [P, D, C.c_double, D, D, D]
    lib.cref_rk4_run.argtypes = [P, D, C.c_int, C.c_double, D, D, D, D, D]
    lib.cref_get_tables.argtypes = [P, D, D]
    lib.cref_threads.restype = C.c_int
    lib.cref_set_threads.argtypes = [C.c_int]
    lib.cref_set_threads.restype = C.c_int
    return lib
