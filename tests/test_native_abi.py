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


def test_encode_launch_counts():
    """nebc7_encode_launches (host logic only, no GPU work): the draft-only
    presets are one kernel; the default preset orders its blocks first (two
    kernels) and runs one; the full-search presets run the staged form: the
    draft kernel, then for each of the 14 passes its list and its kernel,
    the 5 split passes with a preparation, a task and a commit kernel per
    round (3 for the partition searches of modes 1, 3, 7; 4 and 8 for the
    rotations of modes 5 and 4) and a remainder kernel instead."""
    import nebc7_gb300
    from nebc7_gb300 import _native
    from nebc7_gb300._native import Settings
    nebc7_gb300.build()
    lib = _native.load(_native.LIB)
    rounds = [3, 3, 4, 8, 3]
    staged = 1 + 2 * (14 - len(rounds)) + sum(3 + 2 * r for r in rounds)
    cases = {(1, 9, 1, 0, 0, 0): 1, (1, 9, 2, 1, 0, 0): 1, (1, 9, 1, 1, 0, 0): 3,
             (0, 0, 1, 1, 0, 0): 2 + staged, (1, 9, 1, 1, 1, 0): 2 + staged, (1, 9, 1, 1, 0, 1): 2 + staged}
    for st, n in cases.items():
        assert lib.nebc7_encode_launches(ctypes.byref(Settings(*st))) == n, st
    assert lib.nebc7_encode_launches(ctypes.byref(Settings(3, 9, 1, 1, 0, 0))) < 0
