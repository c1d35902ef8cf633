"""The C-ABI library: it builds, loads and exports every symbol include/ma.h declares."""
import os
import re

import pytest

from conftest import ROOT, has_gpu


def _declared():
    with open(os.path.join(ROOT, "include", "ma.h")) as fh:
        src = fh.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ma_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported():
    from mongeampere_gb300 import _lib
    lib = _lib.load()
    declared = _declared()
    assert declared, "no declarations found"
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes table covers the whole header
    assert set(declared) == set(_lib.SIGNATURES)


def test_no_device_is_reported():
    if has_gpu():
        pytest.skip("a GPU is present")
    import ctypes
    from mongeampere_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.ma_ctx_create(0, ctypes.byref(h)) == _lib.MA_ERR_NO_DEVICE
    assert lib.ma_status_string(_lib.MA_EMPTY_CELL).decode() == "a Laguerre cell is empty"


def test_python_api_fails_loudly_without_device():
    if has_gpu():
        pytest.skip("a GPU is present")
    from mongeampere_gb300 import _lib, api
    with pytest.raises(_lib.MaError):
        api.Context(0)
