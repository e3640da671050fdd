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
