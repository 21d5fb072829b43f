"""The C-ABI library loads and exports every entry point include/lcpgrid.h
declares; calls that need a GPU fail cleanly without one."""
import ctypes
import os
import re

import pytest

import lcpgrid
from lcpgrid import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "lcpgrid.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lcp_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    names = declared()
    assert len(names) >= 30
    lib = ctypes.CDLL(_lib.LIB_PATH)
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    assert set(declared()) <= set(_lib.exported_symbols())


def test_version_and_errors():
    assert b"sm_103a" in _lib.lib.lcp_version()
    with pytest.raises(lcpgrid.LCPError):
        _lib.check(_lib.lib.lcp_ucell_get_info(None, None))
    assert b"NULL" in _lib.lib.lcp_last_error()


def test_no_gpu_context_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(lcpgrid.LCPError) as e:
        lcpgrid.Context(0)
    assert e.value.status in (_lib.LCP_EDEVICE, _lib.LCP_EINVAL)
