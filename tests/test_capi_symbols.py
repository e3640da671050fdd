"""The C-ABI library loads and exports every function include/mattohf.h declares (no GPU needed)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(mattohf_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_binding_list():
    from mattohf_gb300 import _capi
    assert sorted(_capi.EXPORTS) == declared_functions()


def test_library_exports_all_symbols(built_lib):
    lib = ctypes.CDLL(os.path.join(ROOT, "mattohf_gb300", "_lib", "libmattohf.so"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_without_gpu(built_lib):
    assert built_lib.mattohf_status_string(0) == b"ok"
    assert built_lib.mattohf_status_string(3) == b"non-finite state"


def test_create_rejects_bad_config_without_gpu(built_lib):
    """Argument validation happens before any CUDA call."""
    from mattohf_gb300 import _capi
    c = _capi.mattohf_config()
    c.NG, c.NK, c.NB, c.NBocc, c.acell = 48, 4, 2, 2, 10.0   # NG not a power of two
    h = ctypes.c_void_p()
    assert built_lib.mattohf_create(ctypes.byref(c), ctypes.byref(h)) == _capi.ERR_ARG
    c.NG, c.NBocc = 64, 3                                      # NBocc > NB
    assert built_lib.mattohf_create(ctypes.byref(c), ctypes.byref(h)) == _capi.ERR_ARG


def test_null_handles_are_rejected_without_gpu(built_lib):
    """Every entry point checks its handle before touching the device."""
    from mattohf_gb300 import _capi
    D = ctypes.POINTER(ctypes.c_double)
    x = (ctypes.c_double * 8)()
    px = ctypes.cast(x, D)
    assert built_lib.mattohf_destroy(None) == _capi.OK
    assert built_lib.mattohf_last_error(None) == b"null context"
    assert built_lib.mattohf_rk4_run(None, 1, ctypes.c_double(0.01), px, px, px, px, px) == _capi.ERR_ARG
    assert built_lib.mattohf_hpsi(None, px, px, 1, ctypes.c_double(0.0), px) == _capi.ERR_ARG
    assert built_lib.mattohf_set_option(None, _capi.OPT_GRAPH, 1) == _capi.ERR_ARG
    assert built_lib.mattohf_batch_destroy(None) == _capi.OK
    assert built_lib.mattohf_batch_set_option(None, _capi.OPT_FOCK_DF64, 1) == _capi.ERR_ARG
    assert built_lib.mattohf_autotune(None, 4, None, None) == _capi.ERR_ARG
    assert built_lib.mattohf_batch_autotune(None, 4, None, None) == _capi.ERR_ARG
    h = ctypes.c_void_p()
    assert built_lib.mattohf_batch_create(0, None, ctypes.byref(h)) == _capi.ERR_ARG


def test_create_validates_geometry_without_gpu(built_lib):
    from mattohf_gb300 import _capi
    z = (ctypes.c_double * 1)(2.0)
    al = (ctypes.c_double * 1)(1.0)
    R = (ctypes.c_double * 1)(0.5)
    K = (ctypes.c_int * 1)(2)                   # species index 2 of 1
    c = _capi.mattohf_config()
    c.NG, c.NK, c.NB, c.NBocc, c.acell = 64, 4, 2, 2, 10.0
    c.nspecies, c.Zeff, c.alpha = 1, ctypes.cast(z, ctypes.POINTER(ctypes.c_double)), \
        ctypes.cast(al, ctypes.POINTER(ctypes.c_double))
    c.nion, c.Rion, c.Kion = 1, ctypes.cast(R, ctypes.POINTER(ctypes.c_double)), \
        ctypes.cast(K, ctypes.POINTER(ctypes.c_int))
    h = ctypes.c_void_p()
    assert built_lib.mattohf_create(ctypes.byref(c), ctypes.byref(h)) == _capi.ERR_ARG
    K[0] = 1
    c.acell = -1.0                              # non-positive cell
    assert built_lib.mattohf_create(ctypes.byref(c), ctypes.byref(h)) == _capi.ERR_ARG
    c.acell = 10.0
    c.NK = 0                                    # no k-points
    assert built_lib.mattohf_create(ctypes.byref(c), ctypes.byref(h)) == _capi.ERR_ARG
    c.NK, c.NB, c.NBocc, c.NG = 1 << 14, 64, 64, 512   # beyond the size limit
    assert built_lib.mattohf_create(ctypes.byref(c), ctypes.byref(h)) == _capi.ERR_ARG
    assert not h.value
