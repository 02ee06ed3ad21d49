"""GPU parity: the CUDA encoder against the reference's outputs (golden
fixtures) and against the CPU oracle port on fresh seeded inputs.

Bit-exact for every 128-bit block and for the integer error sums.  The SSIM
sums are double-precision sums over blocks whose order differs between the
GPU reduction and the CPU job order, so they are compared with a relative
tolerance of 1e-9.
"""

import ctypes
import hashlib

import numpy as np
import pytest

from nebc7_gb300 import synth

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

SSIM_RTOL = 1e-9


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def settings(d, s, dr, no, sl, lin):
    from nebc7_gb300._native import Settings
    return Settings(d, s, dr, no, sl, lin)


def gpu_blocks(native, cells, masks, io, st):
    err = np.zeros(2, np.int64)
    ssim = np.zeros(2, np.float64)
    rc = native.nebc7_encode_blocks_host(cells.ctypes.data, masks.ctypes.data, io.ctypes.data, len(io),
                                         ctypes.byref(st), err.ctypes.data, ssim.ctypes.data)
    return rc, err, ssim


def needs(native, st):
    """Every pass set is built: a build that reports one as unsupported
    (NEBC7_EUNSUPPORTED) fails the case instead of skipping it."""
    z = np.zeros((1, 64), np.uint8)
    rc, _, _ = gpu_blocks(native, z, np.full((1, 64), 255, np.uint8), np.zeros((1, 16), np.uint8), st)
    assert rc != 4, "the library lacks the passes of these settings"
    assert rc == 0


SETS = ["d1s9_draft", "d1s9_draft_restart", "d0s0_draft", "d1s9_normal", "d1s9_slow", "d1s9_normal_restart",
        "d0s0_normal", "d0s0_slow", "d1s0_normal", "d0s9_normal", "d1s9_linear", "d1s9_m6i2", "d1s9_m6i2_restart"]


@pytest.mark.parametrize("name", SETS)
def test_blocks_match_reference(native, golden, blocks_input, name):
    cells, masks, starts = blocks_input
    g = golden["blocks"]["sets"][name]
    st = settings(g["denoise"], g["step"], g["draft"], g["normal"], g["slow"], g["linear"])
    needs(native, st)
    io = np.zeros_like(starts) if g["start"] == "zero" else starts.copy()
    rc, err, ssim = gpu_blocks(native, cells, masks, io, st)
    assert rc == 0
    ref = np.load(GOLDEN / f"blocks_{name}.npz")
    bad = np.nonzero((io != ref["out"]).any(1))[0]
    assert len(bad) == 0, f"{len(bad)} blocks differ, first {bad[:8].tolist()}"
    assert err.tolist() == g["err"]
    assert np.allclose(ssim, g["ssim"], rtol=SSIM_RTOL, atol=0)


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("preset", [(1, 9), (0, 0)])
@pytest.mark.parametrize("passes", [(1, 0, 0), (1, 1, 0), (1, 1, 1), (2, 0, 0)])
def test_blocks_match_oracle(native, port, seed, preset, passes):
    n = 3000
    cells, masks = synth.random_blocks(n, 1000 + seed)
    st = settings(preset[0], preset[1], *passes, 0)
    needs(native, st)
    starts = synth.random_start_blocks(n, 2000 + seed) if seed == 3 else np.zeros((n, 16), np.uint8)
    a = starts.copy()
    b = starts.copy()
    e1, s1 = port.compress_blocks(cells, masks, a, preset[0], preset[1], *passes, 0, threads=16)
    rc, e2, s2 = gpu_blocks(native, cells, masks, b, st)
    assert rc == 0
    bad = np.nonzero((a != b).any(1))[0]
    assert len(bad) == 0, f"{len(bad)} blocks differ, first {bad[:8].tolist()}"
    assert e1.tolist() == e2.tolist()
    assert np.allclose(s1, s2, rtol=SSIM_RTOL, atol=0)


IMAGES = ["cfg1_256_draft", "cfg1_256_default", "cfg2_1024_draft", "cfg2_1024_default", "cfg2_1024_precise",
          "odd_130x98_default", "alpha_256_mask", "alpha_256_retina_precise", "tiny_3x5_default",
          "cfg3_2048_slow", "cfg3_2048_data", "cfg2_1024_m6i2", "alpha_256_m6i2"]


@pytest.mark.parametrize("name", IMAGES)
def test_images_match_reference(native, golden, name):
    """Whole images through the CLI path: full-size SHA-256 of the BC7 payload."""
    from nebc7_gb300 import Preset, encode_image, parse_flags
    g = golden["images"][name]
    o = parse_flags(g["flags"])
    needs(native, settings(g["denoise"], g["step"], int(o["draft"]), int(o["normal"]), int(o["slow"]), int(o["linear"])))
    img = synth.image_for(g["kind"], g["w"], g["h"], g["seed"])
    enc = encode_image(img, g["flags"], Preset(g["denoise"], g["step"]))
    if (GOLDEN / f"image_{name}.npz").exists():
        ref = np.load(GOLDEN / f"image_{name}.npz")["out"]
        bad = np.nonzero((enc.blocks != ref).any(1))[0]
        assert len(bad) == 0, f"{len(bad)} blocks differ, first {bad[:8].tolist()}"
    assert sha(enc.blocks) == g["output_sha256"]
    assert [enc.stats.err_alpha, enc.stats.err_color] == g["err"]
    assert np.allclose([enc.stats.ssim_alpha, enc.stats.ssim_color], g["ssim"], rtol=SSIM_RTOL, atol=0)


def test_decode_matches_oracle(native, port):
    blocks = synth.random_start_blocks(4096, 77)
    out = np.zeros((4096, 64), np.uint8)
    assert native.nebc7_decode_blocks_host(blocks.ctypes.data, out.ctypes.data, 4096) == 0
    assert np.array_equal(out, port.decompress_blocks(blocks))


def test_bc7core_vtable_and_process_texture(native, port):
    """The reference-shaped entry points: IBc7Core.pCompress over WorkerItems
    (accumulating) and ProcessTexture over a texture."""
    from nebc7_gb300._native import BlockSSIM, IBc7Core, WorkerItem
    core = IBc7Core()
    assert native.nebc7_GetBc7Core(ctypes.byref(core))
    assert native.nebc7_set_preset(1, 9) == 0
    core.pInitTables(True, False, False, False)
    img = synth.photo_like(64, 32, 5)
    mask = np.full_like(img, 255)
    stride = 64 * 4
    n = 16 * 8
    out = np.zeros((n, 16), np.uint8)
    items = (WorkerItem * n)()
    for k in range(n):
        bx, by = k % 16, k // 16
        off = by * 4 * stride + bx * 16
        items[k]._Output = out.ctypes.data + 16 * k
        items[k]._Cell = img.ctypes.data + off
        items[k]._Mask = mask.ctypes.data + off
    ea = ctypes.c_int64(5)
    ec = ctypes.c_int64(7)
    q = BlockSSIM(1.0, 2.0)
    core.pCompress(items, ctypes.cast(ctypes.byref(items, ctypes.sizeof(WorkerItem) * n), ctypes.POINTER(WorkerItem)),
                   stride, ctypes.byref(ea), ctypes.byref(ec), ctypes.byref(q))
    ref = np.zeros((n, 16), np.uint8)
    e, s = port.compress_texture(ref, img, mask, 1, 9, 1, 0, 0, 0)
    assert np.array_equal(out, ref)
    assert ea.value == 5 + e[0] and ec.value == 7 + e[1]   # pCompress adds
    # ProcessTexture assigns
    out2 = np.zeros((n, 16), np.uint8)
    native.nebc7_ProcessTexture(out2.ctypes.data, img.ctypes.data, mask.ctypes.data, stride, 64, 32,
                                ctypes.cast(core.pCompress, ctypes.c_void_p), 16, ctypes.byref(ea), ctypes.byref(ec),
                                ctypes.byref(q))
    assert np.array_equal(out2, ref)
    assert ea.value == e[0] and ec.value == e[1]


def test_invalid_arguments_are_rejected(native):
    from nebc7_gb300._native import Settings
    st = Settings(2, 9, 1, 0, 0, 0)
    z = np.zeros((1, 64), np.uint8)
    io = np.zeros((1, 16), np.uint8)
    assert native.nebc7_encode_blocks_host(z.ctypes.data, z.ctypes.data, io.ctypes.data, 1, ctypes.byref(st), None, None) == 1
    st = Settings(1, 9, 1, 0, 0, 0)
    assert native.nebc7_encode_host(io.ctypes.data, z.ctypes.data, None, 24, 6, 4, ctypes.byref(st), None, None) == 1
    assert native.nebc7_set_preset(3, 0) == 1
