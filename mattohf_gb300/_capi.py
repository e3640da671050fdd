"""ctypes binding of the C ABI declared in ``include/mattohf.h``.

The shared library is built in-tree (``mattohf_gb300/_lib/libmattohf.so``).
There is no fallback: if the library is missing or cannot be loaded the
import raises, so the CUDA path is the only path.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmattohf.so")

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_NONFINITE = 3
ERR_TIMEOUT = 4
ERR_NOTCONV = 5
ERR_ALLOC = 6
ERR_STATE = 7
ERR_TOO_LARGE = 8

OPT_GRAPH = 1
OPT_FOCK_CHUNKS = 2
OPT_KERNEL_TIMING = 3
OPT_SYMMETRIC = 4
OPT_L2_FLUSH = 5
OPT_FOCK_DF64 = 6
OPT_SYM_TILE = 7
OPT_SMALL_STAGES = 8
OPT_SMALL_CTAS = 9

# every symbol include/mattohf.h declares
EXPORTS = [
    "mattohf_create", "mattohf_destroy", "mattohf_last_error", "mattohf_status_string",
    "mattohf_set_option", "mattohf_get_grids", "mattohf_get_coulomb", "mattohf_get_vion",
    "mattohf_set_vion", "mattohf_set_orbitals", "mattohf_get_orbitals", "mattohf_init_wf",
    "mattohf_gram_schmidt", "mattohf_hpsi", "mattohf_hpsi_device", "mattohf_fock",
    "mattohf_hpsi_kslice_device", "mattohf_observables_kslice_device",
    "mattohf_kinetic", "mattohf_density", "mattohf_observables", "mattohf_rk4_step",
    "mattohf_rk4_run", "mattohf_last_run_timing", "mattohf_gs_run", "mattohf_eps",
    "mattohf_synchronize", "mattohf_diag_fp64_peak", "mattohf_diag_dmma_peak", "mattohf_fock_noalloc",
    "mattohf_batch_create", "mattohf_batch_destroy", "mattohf_batch_last_error", "mattohf_batch_run",
    "mattohf_batch_rk4_run", "mattohf_batch_last_run_ms", "mattohf_adjoint", "mattohf_adjoint_timing",
    "mattohf_fourier", "mattohf_vck", "mattohf_te_step", "mattohf_batch_set_option", "mattohf_autotune",
    "mattohf_batch_autotune", "mattohf_ion_param_grad", "mattohf_batch_adjoint",
]


class mattohf_config(C.Structure):
    _fields_ = [
        ("NG", C.c_int), ("NK", C.c_int), ("NB", C.c_int), ("NBocc", C.c_int),
        ("acell", C.c_double), ("functional_hf", C.c_int), ("device", C.c_int),
        ("nspecies", C.c_int), ("Zeff", C.POINTER(C.c_double)), ("alpha", C.POINTER(C.c_double)),
        ("nion", C.c_int), ("Rion", C.POINTER(C.c_double)), ("Kion", C.POINTER(C.c_int)),
    ]


_lib = None


def load(path: str = LIB_PATH):
    """Load the library once; raise if it is absent (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -m mattohf_gb300.build` "
            "(the CUDA library is the only implementation)")
    lib = C.CDLL(path)
    P = C.c_void_p
    D = C.POINTER(C.c_double)
    I = C.c_int
    sig = {
        "mattohf_create": ([C.POINTER(mattohf_config), C.POINTER(P)], I),
        "mattohf_destroy": ([P], I),
        "mattohf_last_error": ([P], C.c_char_p),
        "mattohf_status_string": ([I], C.c_char_p),
        "mattohf_set_option": ([P, I, C.c_longlong], I),
        "mattohf_get_grids": ([P, D, D, D, D], I),
        "mattohf_get_coulomb": ([P, D, D], I),
        "mattohf_get_vion": ([P, D], I),
        "mattohf_set_vion": ([P, D], I),
        "mattohf_set_orbitals": ([P, D], I),
        "mattohf_get_orbitals": ([P, D], I),
        "mattohf_init_wf": ([P], I),
        "mattohf_gram_schmidt": ([P], I),
        "mattohf_hpsi": ([P, D, D, I, C.c_double, D], I),
        "mattohf_hpsi_device": ([P, P, P, I, C.c_double, P], I),
        "mattohf_hpsi_kslice_device": ([P, P, I, I, P, I, C.c_double, I, P], I),
        "mattohf_observables_kslice_device": ([P, P, I, I, P, C.c_double, D, D], I),
        "mattohf_fock": ([P, D, D, I, D], I),
        "mattohf_kinetic": ([P, D, I, C.c_double, D], I),
        "mattohf_density": ([P, D, D, D], I),
        "mattohf_observables": ([P, C.c_double, D, D, D, D], I),
        "mattohf_rk4_step": ([P, C.c_double, C.c_double, C.c_double], I),
        "mattohf_rk4_run": ([P, I, C.c_double, D, D, D, D, D], I),
        "mattohf_last_run_timing": ([P, D, D, C.POINTER(C.c_int)], I),
        "mattohf_autotune": ([P, I, C.POINTER(C.c_int), D], I),
        "mattohf_batch_autotune": ([P, I, C.POINTER(C.c_int), D], I),
        "mattohf_gs_run": ([P, I, I, D, D, D, D, D], I),
        "mattohf_eps": ([P, D, D], I),
        "mattohf_synchronize": ([P], I),
        "mattohf_diag_dmma_peak": ([I, D], I),
        "mattohf_diag_fp64_peak": ([I, D], I),
        "mattohf_fock_noalloc": ([I, I, I, I, I, P, P, P, P, P], I),
        "mattohf_batch_create": ([I, C.POINTER(mattohf_config), C.POINTER(P)], I),
        "mattohf_batch_destroy": ([P], I),
        "mattohf_batch_last_error": ([P], C.c_char_p),
        "mattohf_batch_run": ([P, I], P),
        "mattohf_batch_rk4_run": ([P, I, D, D, D, D, D, D], I),
        "mattohf_batch_last_run_ms": ([P, D], I),
        "mattohf_batch_set_option": ([P, I, C.c_longlong], I),
        "mattohf_adjoint": ([P, I, I, C.c_double, D, I, D, D, D], I),
        "mattohf_adjoint_timing": ([P, D, D], I),
        "mattohf_ion_param_grad": ([P, D, D, D, D], I),
        "mattohf_batch_adjoint": ([P, I, I, D, D, I, D, D, D], I),
        "mattohf_vck": ([P, D, I, D], I),
        "mattohf_te_step": ([P, I, C.c_double, C.c_double], I),
        "mattohf_fourier": ([I, I, D, D, C.c_double, D, D, D, I, C.c_double, C.c_double, D], I),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib
