"""The driver's steps on the device -- padding and outline masks, the /bad
glitch map and the /map partition visualisation -- against the oracle
(GPU)."""

import ctypes

import numpy as np
import pytest

from nebc7_gb300 import synth
from oracle import pytools

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.device("cuda", 0))


@pytest.mark.parametrize("w,h", [(3, 5), (130, 98), (64, 64), (257, 31)])
@pytest.mark.parametrize("radius", [-1, 1, 2])
def test_prepare_matches_oracle(native, port, w, h, radius):
    torch = pytest.importorskip("torch")
    img = synth.alpha_blobs(w, h, 3)
    want_pad, want_mask = port.prepare(img, radius)
    ph, pw = want_pad.shape[:2]
    d_src = _dev(torch, img)
    d_pad = torch.zeros(ph * pw * 4, dtype=torch.uint8, device="cuda")
    d_mask = torch.zeros_like(d_pad)
    assert native.nebc7_prepare_device(d_src.data_ptr(), w * 4, w, h, d_pad.data_ptr(), d_mask.data_ptr(), radius, None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_pad.cpu().numpy().reshape(ph, pw, 4), want_pad)
    assert np.array_equal(d_mask.cpu().numpy().reshape(ph, pw, 4), want_mask)


@pytest.mark.parametrize("linear", [0, 1])
def test_bad_block_map_matches_oracle(native, port, linear):
    torch = pytest.importorskip("torch")
    from nebc7_gb300.api import outline_mask, pad_texture
    from nebc7_gb300._native import Settings
    img = pad_texture(synth.alpha_blobs(96, 64, 8))
    mask = outline_mask(img, 1)
    h, w = img.shape[:2]
    d_img, d_mask = _dev(torch, img), _dev(torch, mask)
    d_blocks = torch.zeros((h // 4) * (w // 4) * 16, dtype=torch.uint8, device="cuda")
    st = Settings(1, 9, 1, 0, 0, linear)     # draft: leaves visible glitches to find
    assert native.nebc7_encode_device(d_blocks.data_ptr(), d_img.data_ptr(), d_mask.data_ptr(), w * 4, w, h,
                                      ctypes.byref(st), None, None, None) == 0
    d_dec = torch.zeros_like(d_img)
    assert native.nebc7_decode_device(d_blocks.data_ptr(), d_dec.data_ptr(), w * 4, w, h, None) == 0
    d_out = torch.zeros_like(d_img)
    assert native.nebc7_bad_blocks_device(d_img.data_ptr(), d_dec.data_ptr(), d_mask.data_ptr(), w * 4, w, h, linear,
                                          d_out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    want = pytools.bad_blocks(img, d_dec.cpu().numpy(), mask, bool(linear))
    got = d_out.cpu().numpy()
    assert np.array_equal(got, want)
    assert got.any() and not np.array_equal(got, img)   # some blocks flagged, not all


def test_partition_map_matches_oracle(native, port):
    torch = pytest.importorskip("torch")
    from nebc7_gb300.api import pad_texture
    from nebc7_gb300._native import Settings
    parts = [synth.random_start_blocks(2048, 5)]
    for preset in [(1, 9, 1, 1, 1, 0), (0, 0, 1, 1, 0, 0)]:
        img = pad_texture(synth.alpha_blobs(64, 64, 1))
        d_img = _dev(torch, img)
        d_blocks = torch.zeros(16 * 16 * 16, dtype=torch.uint8, device="cuda")
        assert native.nebc7_encode_device(d_blocks.data_ptr(), d_img.data_ptr(), None, 256, 64, 64,
                                          ctypes.byref(Settings(*preset)), None, None, None) == 0
        parts.append(d_blocks.cpu().numpy().reshape(-1, 16))
    blocks = np.concatenate(parts + [np.tile(np.array([[0x40] + [0] * 15], np.uint8), (4, 1))])
    d_in = _dev(torch, blocks)
    d_out = torch.zeros_like(d_in)
    assert native.nebc7_partition_map_device(d_in.data_ptr(), d_out.data_ptr(), len(blocks), None) == 0
    torch.cuda.synchronize()
    got = d_out.cpu().numpy().reshape(-1, 16)
    assert np.array_equal(got, pytools.partition_map(blocks))
    # and the map decodes (device) like the oracle's decoder
    out = np.zeros((len(got), 64), np.uint8)
    assert native.nebc7_decode_blocks_host(np.ascontiguousarray(got).ctypes.data, out.ctypes.data, len(got)) == 0
    assert np.array_equal(out, port.decompress_blocks(got))


REF_CLI = ["tools_alpha_96x64_draft", "tools_alpha_96x64_data", "tools_photo_64_default", "tools_alpha_62x46_slow"]


@pytest.mark.parametrize("name", REF_CLI)
def test_device_bad_and_map_match_reference_cli(native, port, golden, name):
    """The device /bad and /map steps on the reference CLI's own blocks give
    the images the reference CLI wrote (tests/golden/tools_*.npz)."""
    torch = pytest.importorskip("torch")
    from nebc7_gb300.api import parse_flags
    from conftest import GOLDEN
    g = golden["tools"][name]
    f = np.load(GOLDEN / f"{name}.npz")
    o = parse_flags(g["flags"])
    img = synth.image_for(g["kind"], g["w"], g["h"], g["seed"])
    padded, mask = port.prepare(img, o["radius"] if o["mask"] else -1)
    ph, pw = padded.shape[:2]
    d_img = _dev(torch, padded)
    d_mask = _dev(torch, mask) if o["mask"] else None
    d_blocks = _dev(torch, f["blocks"])
    d_dec = torch.zeros_like(d_img)
    assert native.nebc7_decode_device(d_blocks.data_ptr(), d_dec.data_ptr(), pw * 4, pw, ph, None) == 0
    d_bad = torch.zeros_like(d_img)
    assert native.nebc7_bad_blocks_device(d_img.data_ptr(), d_dec.data_ptr(),
                                          d_mask.data_ptr() if d_mask is not None else None, pw * 4, pw, ph,
                                          int(o["linear"]), d_bad.data_ptr(), None) == 0
    d_vis = torch.zeros_like(d_blocks)
    assert native.nebc7_partition_map_device(d_blocks.data_ptr(), d_vis.data_ptr(), len(f["blocks"]), None) == 0
    d_map = torch.zeros_like(d_img)
    assert native.nebc7_decode_device(d_vis.data_ptr(), d_map.data_ptr(), pw * 4, pw, ph, None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_bad.cpu().numpy().reshape(ph, pw, 4), f["bad"])
    assert np.array_equal(d_map.cpu().numpy().reshape(ph, pw, 4), f["map"])
