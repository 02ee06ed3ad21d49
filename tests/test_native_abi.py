"""CPU tests: the C-ABI library builds for sm_103a, loads, and exports every
symbol include/nebc7_gb300.h declares (no GPU work is launched)."""

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "nebc7_gb300.h").read_text()
    return sorted(set(re.findall(r"^\w[\w\s\*]*?\b(nebc7_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "nebc7_GetBc7Core" in syms and "nebc7_ProcessTexture" in syms
    assert len(syms) >= 10


def test_library_exports_declared_symbols():
    import nebc7_gb300
    from nebc7_gb300 import _native
    nebc7_gb300.build()
    lib = ctypes.CDLL(str(_native.LIB))
    for s in declared_symbols():
        assert hasattr(lib, s), s
    assert set(declared_symbols()) == set(_native.SIGNATURES)


def test_load_fails_loudly_without_library(tmp_path):
    from nebc7_gb300 import _native
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _native.load(tmp_path / "missing.so")
