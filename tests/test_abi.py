"""CPU checks of the C ABI: the library loads and exports every symbol include/warp_gb300.h declares
(no compute call is made without a GPU)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "warp_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def _lib_path():
    from warp_gb300 import _native

    return _native.LIB_PATH


def test_header_declares_functions():
    names = declared_functions()
    assert "gb_bsr_matrix_from_triplets_device" in names
    assert "gb_bsr_mv" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    path = _lib_path()
    if not os.path.exists(path):
        pytest.skip("library not built")
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_header():
    from warp_gb300 import _native, fem  # noqa: F401  (fem registers its entry points)

    bound = set(_native.exported_names())
    missing = [n for n in declared_functions() if n not in bound]
    assert not missing, missing


def test_library_reports_version_without_gpu():
    path = _lib_path()
    if not os.path.exists(path):
        pytest.skip("library not built")
    lib = ctypes.CDLL(path)
    assert lib.gb_version() == 100
    lib.gb_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.gb_last_error(), bytes)


def test_convnet_launch_rejects_bad_arguments_without_gpu():
    """The whole-network conv entry point checks its arguments before any CUDA call: these return
    GB_ERR_INVALID on a machine without a GPU."""
    from warp_gb300 import _native as N

    path = _lib_path()
    if not os.path.exists(path):
        pytest.skip("library not built")
    L = N.lib()
    # work items: columns of 252 padded rows over an x-slab's interior rows, times nx
    assert L.gb_convnet_tc_items(97, 97, 97) == -(-(96 * 99 + 97) // 252) * 97
    assert L.gb_convnet_tc_items(9, 9, 9) == 9
    assert L.gb_convnet_tc_items(0, 9, 9) == 0
    bufs = (ctypes.c_void_p * 4)(16, 32, 48, 64)
    wts = (ctypes.c_void_p * 4)(16, 32, 48, 64)
    one = ctypes.c_void_p(16)

    def call(nlayers=4, ncomp=1, act=bufs, wt=wts, w=one, flags=one, status=one):
        return L.gb_convnet_fwd_tc(9, 9, 9, ncomp, nlayers, act, wt, w, one, one, None, None, 0.6, flags, one,
                                   status, None)

    invalid = -1
    assert call(nlayers=5) == invalid
    assert call(nlayers=1) == invalid
    assert call(ncomp=2) == invalid
    assert call(w=None) == invalid
    assert call(flags=None) == invalid
    assert call(status=None) == invalid
    assert call(act=(ctypes.c_void_p * 4)(16, 33, 48, 64)) == invalid  # misaligned activation buffer
    assert call(wt=(ctypes.c_void_p * 4)(16, 32, 0, 64)) == invalid    # missing weights
    assert b"convnet_fwd_tc" in L.gb_last_error()


def test_product_does_not_import_oracle():
    pkg = os.path.join(ROOT, "warp_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh")):
                src = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
