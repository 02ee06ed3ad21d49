"""CPU tests: the oracle port against the reference's own outputs.

The golden fixtures were produced by the reference encoder compiled from its
sources (tests/golden/make_golden.py); these tests pin the scalar port that
the GPU parity tests use as their checker.
"""

import hashlib

import numpy as np
import pytest

from nebc7_gb300 import synth

from conftest import GOLDEN


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_synthetic_inputs_reproduce(golden, blocks_input):
    cells, masks, starts = blocks_input
    assert sha(cells) == golden["blocks"]["cells_sha256"]
    assert sha(masks) == golden["blocks"]["masks_sha256"]
    assert sha(starts) == golden["blocks"]["starts_sha256"]
    for name, g in golden["images"].items():
        if g["w"] * g["h"] > 1024 * 1024:
            continue
        img = synth.image_for(g["kind"], g["w"], g["h"], g["seed"])
        assert sha(img) == g["input_sha256"], name


SETS = ["d1s9_draft", "d1s9_normal", "d1s9_slow", "d1s9_normal_restart", "d1s9_draft_restart",
        "d0s0_draft", "d0s0_normal", "d0s0_slow", "d1s0_normal", "d0s9_normal", "d1s9_linear",
        "d1s9_m6i2", "d1s9_m6i2_restart"]


@pytest.mark.parametrize("name", SETS)
def test_port_blocks_match_reference(port, golden, blocks_input, name):
    cells, masks, starts = blocks_input
    g = golden["blocks"]["sets"][name]
    io = np.zeros_like(starts) if g["start"] == "zero" else starts.copy()
    err, ssim = port.compress_blocks(cells, masks, io, g["denoise"], g["step"], g["draft"], g["normal"], g["slow"],
                                     g["linear"], threads=8)
    ref = np.load(GOLDEN / f"blocks_{name}.npz")
    assert np.array_equal(io, ref["out"]), f"{int(np.count_nonzero((io != ref['out']).any(1)))} blocks differ"
    assert err.tolist() == g["err"]
    assert ssim.tolist() == g["ssim"]  # same job order, same double sums


@pytest.mark.parametrize("name", ["cfg1_256_default", "cfg1_256_draft", "cfg2_1024_draft", "cfg2_1024_default",
                                  "odd_130x98_default", "alpha_256_mask", "tiny_3x5_default", "cfg2_1024_m6i2",
                                  "alpha_256_m6i2"])
def test_port_images_match_reference(port, golden, name):
    from nebc7_gb300.api import parse_flags
    g = golden["images"][name]
    img = synth.image_for(g["kind"], g["w"], g["h"], g["seed"])
    o = parse_flags(g["flags"])
    padded, mask = port.prepare(img, o["radius"] if o["mask"] else -1)
    out = np.zeros((padded.shape[0] // 4 * (padded.shape[1] // 4), 16), np.uint8)
    err, ssim = port.compress_texture(out, padded, mask, g["denoise"], g["step"], int(o["draft"]), int(o["normal"]),
                                      int(o["slow"]), int(o["linear"]), threads=8)
    assert sha(out) == g["output_sha256"]
    assert err.tolist() == g["err"]
    assert np.allclose(ssim, g["ssim"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("radius", [-1, 1, 2])
@pytest.mark.parametrize("size", [(3, 5), (130, 98), (64, 64)])
def test_host_padding_and_mask_match_port(port, radius, size):
    from nebc7_gb300.api import outline_mask, pad_texture
    img = synth.alpha_blobs(size[0], size[1], 7)
    padded, mask = port.prepare(img, radius)
    assert np.array_equal(pad_texture(img), padded)
    if radius >= 0:
        assert np.array_equal(outline_mask(padded, radius), mask)


def test_port_tables_match_reference():
    import ctypes
    from oracle.pyoracle import REF_DIR, Port, Reference
    if not (REF_DIR / "libnebc7_ref_d1s9.so").exists():
        pytest.skip("reference build not present (x86 host with the reference sources only)")
    p = Port()
    for d, s in ((1, 9), (0, 0)):
        r = Reference(d, s)
        z = np.zeros(64, np.uint8)
        r.compress_blocks(z, np.full(64, 255, np.uint8), np.zeros((1, 16), np.uint8), 1, 0, 0, 0, 1)
        for tid in range(14):
            n1, n2 = ctypes.c_int(), ctypes.c_int()
            a = r.lib.nebc7_ref_table(tid, ctypes.byref(n1))
            b = p.lib.nebc7_oracle_table(d, tid, ctypes.byref(n2))
            assert n1.value == n2.value
            assert ctypes.string_at(a, n1.value) == ctypes.string_at(b, n2.value), (d, tid)


def test_port_mode6index2_only_run(port, blocks_input):
    """The "Mode6Index2 fast" run (doDraft 2; the reference's m6i2 variant,
    oracle/ref_m6i2_only.cpp, pins it above): every block stays the starting
    block or becomes a mode 6 block, and the error is never below the full
    draft chain's."""
    cells, masks, _ = blocks_input
    io6 = np.zeros((len(cells), 16), np.uint8)
    e6, _ = port.compress_blocks(cells, masks, io6, 1, 9, 2, 0, 0, 0, threads=4)
    iod = np.zeros_like(io6)
    ed, _ = port.compress_blocks(cells, masks, iod, 1, 9, 1, 0, 0, 0, threads=4)
    assert np.all((io6[:, 0] & 0x7F) == 0x40)          # mode 6 (or the zero mode-6 start)
    assert int(e6.sum()) >= int(ed.sum())
    assert not np.array_equal(io6, iod)
