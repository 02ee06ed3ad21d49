"""CPU tests of bench.py's report arithmetic (no GPU)."""

import json

import pytest

from conftest import ROOT


def _prof(**kw):
    import bench
    p = {"warp_inst_per_launch": 2_480_000_000, "summary": "KEncode_photo1024_default_full.md",
         "source_sha": bench.source_sha()}
    p.update(kw)
    return p


def test_issue_roofline_arithmetic():
    import bench
    r = bench.issue_roofline(_prof(), 5.6, 2070.0, 152)
    assert r["peak"] == pytest.approx(4 * 152 * 2.070)            # G warp-instructions/s
    assert r["achieved"] == pytest.approx(2.48e9 / 5.6e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["source"] == "profiles/KEncode_photo1024_default_full.md"


def test_issue_roofline_refuses_a_capture_of_other_sources():
    import bench
    assert bench.issue_roofline(_prof(source_sha="0" * 16), 5.6, 2070.0, 152) is None
    assert bench.issue_roofline(_prof(source_sha=None), 5.6, 2070.0, 152) is None


@pytest.mark.parametrize("prof,ms,mhz", [(None, 5.6, 2070.0), ({"summary": "x"}, 5.6, 2070.0),
                                         ({"warp_inst_per_launch": 1, "summary": "x"}, 5.6, None),
                                         ({"warp_inst_per_launch": 1, "summary": "x"}, 0.0, 2070.0)])
def test_issue_roofline_needs_capture_clock_and_time(prof, ms, mhz):
    import bench
    if prof is not None:
        prof = dict(prof, source_sha=bench.source_sha())
    assert bench.issue_roofline(prof, ms, mhz, 152) is None


def test_committed_captures_have_the_fields_the_bench_reads():
    """Every workload's capture has its per-encode instructions and DRAM bytes
    and names its summary; the single-kernel workload's full-set capture also
    has the issue and pipe utilisation.  The captures are of one build."""
    profs = json.loads((ROOT / "profiles" / "kencode_ncu.json").read_text())
    assert "photo1024_default" in profs
    for prof in profs.values():
        for key in ("dram_bytes_per_launch", "warp_inst_per_launch", "summary", "source_sha"):
            assert key in prof
        assert prof["warp_inst_per_launch"] > 0
        assert (ROOT / "profiles" / prof["summary"]).exists()
    for key in ("sm_issue_active_pct_elapsed", "pipe_alu_pct_active", "pipe_fma_pct_active"):
        assert key in profs["photo1024_default"]
    assert len({p["source_sha"] for p in profs.values()}) == 1


def test_simd_equivalent_scales_the_port_by_the_calibration():
    import bench
    cal = json.loads((ROOT / "oracle" / "cpu_calibration.json").read_text())
    for name, w in cal["workloads"].items():
        r = bench.simd_equivalent(name, 2.0)
        assert r["value"] == pytest.approx(2.0 * w["port_time_over_reference"])
        assert w["outputs_identical"]
    assert bench.simd_equivalent("no_such_workload", 2.0) is None


def test_work_roofline_arithmetic(tmp_path, monkeypatch):
    import bench
    f = ROOT / "oracle" / "work_counts.json"
    if not f.exists():
        pytest.skip("no work counts committed")
    w = json.loads(f.read_text())["workloads"]
    name = sorted(w)[0]
    r = bench.work_roofline(name, 5.0, 2070.0, 152)
    assert r["peak"] == pytest.approx(128 * 152 * 2.070e9 / 1e12)
    assert r["achieved"] == pytest.approx(w[name]["int_ops"] / 5e-3 / 1e12)
