"""CPU test: include/nebc7_gb300.h's WorkerItem, BlockSSIM and IBc7Core have
the reference's layout (src/Bc7Core.h:25-35, :294-322), checked by
static_asserts in tests/abi/layout_check.cpp compiled against the
reference's own header.  Skipped where the reference sources are absent."""

import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_structures_match_reference_header():
    sys.path.insert(0, str(ROOT))
    from __graft_entry__ import reference_sources
    src = reference_sources()
    if src is None:
        pytest.skip("reference sources not present")
    gxx = shutil.which("g++")
    if gxx is None or "x86" not in subprocess.run(["uname", "-m"], capture_output=True, text=True).stdout:
        pytest.skip("the reference's headers need an x86-64 g++ (SIMD intrinsics)")
    cmd = [gxx, "-std=c++17", "-fsyntax-only", "-mavx2", "-mfma", "-mbmi", "-mbmi2", "-mlzcnt", "-mpopcnt", "-w",
           "-DOPTION_LIBRARY", "-include", str(ROOT / "oracle" / "ref_shim.h"), f"-I{src}", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "abi" / "layout_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
