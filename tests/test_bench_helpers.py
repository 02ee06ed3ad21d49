"""CPU tests of bench.py's report arithmetic (no GPU)."""

import json

import pytest

from conftest import ROOT


def test_issue_roofline_arithmetic():
    import bench
    prof = {"warp_inst_per_launch": 2_480_000_000, "summary": "KEncode_photo1024_default_full.md"}
    r = bench.issue_roofline(prof, 5.6, 2070.0, 152)
    assert r["peak"] == pytest.approx(4 * 152 * 2.070)            # G warp-instructions/s
    assert r["achieved"] == pytest.approx(2.48e9 / 5.6e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["source"] == "profiles/KEncode_photo1024_default_full.md"


@pytest.mark.parametrize("prof,ms,mhz", [(None, 5.6, 2070.0), ({"summary": "x"}, 5.6, 2070.0),
                                         ({"warp_inst_per_launch": 1, "summary": "x"}, 5.6, None),
                                         ({"warp_inst_per_launch": 1, "summary": "x"}, 0.0, 2070.0)])
def test_issue_roofline_needs_capture_clock_and_time(prof, ms, mhz):
    import bench
    assert bench.issue_roofline(prof, ms, mhz, 152) is None


def test_committed_capture_has_the_fields_the_bench_reads():
    prof = json.loads((ROOT / "profiles" / "kencode_ncu.json").read_text())["photo1024_default"]
    for key in ("dram_bytes_per_launch", "sm_issue_active_pct_elapsed", "pipe_alu_pct_active", "pipe_fma_pct_active",
                "warp_inst_per_launch", "summary"):
        assert key in prof
    assert (ROOT / "profiles" / prof["summary"]).exists()
