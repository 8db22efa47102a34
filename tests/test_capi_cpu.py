"""CPU-side checks of the C ABI library: it loads and exports every declared symbol."""

import ctypes

from sfem_gb300 import capi


def test_library_exports_declared_symbols():
    lib = capi.load()
    names = capi.declared_symbols()
    assert "cu_laplacian_apply" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_string():
    lib = capi.load()
    assert b"sm_103a" in lib.sfem_gb300_version()
    assert isinstance(capi.last_error(), str)
