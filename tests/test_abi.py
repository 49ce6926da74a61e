"""The C ABI: the library builds, loads without a GPU, and exports every
function include/sl3dgpu.h declares."""

import ctypes

import pytest


@pytest.fixture(scope="module")
def built():
    import __graft_entry__

    __graft_entry__.build()
    from sl3dpp_gb300 import _lib

    return _lib


def test_library_exports_every_declared_symbol(built):
    L = ctypes.CDLL(str(built.LIBRARY_PATH))
    names = built.exported_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_error_text_without_a_gpu(built):
    L = built.lib()
    assert b"sm_103a" in L.sl3dgpu_version()
    # argument checks answer before any device work
    assert L.sl3dgpu_band_cholesky_factor(None, -1, 3) == built.ERR_ARGUMENT
    assert b"negative" in L.sl3dgpu_last_error()
