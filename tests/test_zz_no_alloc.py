"""nebc7_encode_device_noalloc against nebc7_encode_device (GPU).

The allocation-free entry keeps its scratch in one fixed device array of the
library.  This file is collected last, so it runs both alone and after every
other GPU test has used the library (tables built, staging slots cached).
Two calls in a row must each give the same blocks and the same error / SSIM
sums as the allocating entry point.
"""

import ctypes

import numpy as np
import pytest

from nebc7_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_BLOCKS = 65536   # capacity of the entry's fixed scratch (a 1024x1024 texture)
SSIM_RTOL = 1e-9     # the two paths reduce the same per-block values in the same order


def _settings(d, s, draft, normal, slow):
    from nebc7_gb300._native import Settings
    return Settings(d, s, draft, normal, slow, 0)


def _encode_reference_entry(native, torch, img, mask, st):
    h, w = img.shape[:2]
    dev = torch.device("cuda", 0)
    d_img = torch.from_numpy(img).to(dev)
    d_mask = torch.from_numpy(mask).to(dev) if mask is not None else None
    d_dst = torch.zeros((h // 4) * (w // 4) * 16, dtype=torch.uint8, device=dev)
    errs = np.zeros(2, np.int64)
    ssim = np.zeros(2, np.float64)
    rc = native.nebc7_encode_device(d_dst.data_ptr(), d_img.data_ptr(), d_mask.data_ptr() if d_mask is not None else None,
                                    w * 4, w, h, ctypes.byref(st), errs.ctypes.data, ssim.ctypes.data,
                                    torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 0
    return d_dst.cpu().numpy(), errs, ssim


def _encode_noalloc(native, torch, img, mask, st, with_sums=True):
    h, w = img.shape[:2]
    dev = torch.device("cuda", 0)
    d_img = torch.from_numpy(img).to(dev)
    d_mask = torch.from_numpy(mask).to(dev) if mask is not None else None
    d_dst = torch.zeros((h // 4) * (w // 4) * 16, dtype=torch.uint8, device=dev)
    d_sums = torch.zeros(4, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = native.nebc7_encode_device_noalloc(d_dst.data_ptr(), d_img.data_ptr(),
                                            d_mask.data_ptr() if d_mask is not None else None, w * 4, w, h,
                                            ctypes.byref(st), d_sums.data_ptr() if with_sums else None,
                                            stream.cuda_stream)
    assert rc == 0
    stream.synchronize()
    raw = d_sums.cpu().numpy()
    return d_dst.cpu().numpy(), raw[:2].copy(), raw[2:].view(np.float64).copy()


CASES = {
    "photo256_default": ("photo_like", 256, 256, 11, None, (1, 9, 1, 1, 0)),
    "photo256_precise": ("photo_like", 256, 128, 12, None, (0, 0, 1, 1, 0)),
    "alpha256_slow_mask": ("alpha_blobs", 256, 256, 13, 1, (1, 9, 1, 1, 1)),
    "photo256_draft": ("photo_like", 128, 256, 14, None, (1, 9, 1, 0, 0)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_matches_encode_device_twice(native, name):
    torch = pytest.importorskip("torch")
    from nebc7_gb300.api import outline_mask
    kind, w, h, seed, radius, preset = CASES[name]
    img = synth.image_for(kind, w, h, seed)
    mask = outline_mask(img, radius) if radius is not None else None
    st = _settings(*preset)
    assert native.nebc7_init_device(preset[0]) == 0
    ref_blocks, ref_errs, ref_ssim = _encode_reference_entry(native, torch, img, mask, st)
    for _ in range(2):
        blocks, errs, ssim = _encode_noalloc(native, torch, img, mask, st)
        assert np.array_equal(blocks, ref_blocks)
        assert errs.tolist() == ref_errs.tolist()
        assert np.allclose(ssim, ref_ssim, rtol=SSIM_RTOL, atol=0)
    blocks, _, _ = _encode_noalloc(native, torch, img, mask, st, with_sums=False)
    assert np.array_equal(blocks, ref_blocks)


def test_noalloc_at_its_exact_capacity(native):
    """A 1024x1024 texture fills the fixed scratch exactly (65536 blocks): the
    last block's result sits at the end of the array."""
    torch = pytest.importorskip("torch")
    img = synth.image_for("photo_like", 1024, 1024, 15)
    assert (1024 // 4) * (1024 // 4) == MAX_BLOCKS
    for preset in ((1, 9, 1, 0, 0), (1, 9, 1, 1, 0)):
        st = _settings(*preset)
        assert native.nebc7_init_device(preset[0]) == 0
        ref_blocks, ref_errs, ref_ssim = _encode_reference_entry(native, torch, img, None, st)
        for _ in range(2):
            blocks, errs, ssim = _encode_noalloc(native, torch, img, None, st)
            assert np.array_equal(blocks, ref_blocks)
            assert errs.tolist() == ref_errs.tolist()
            assert np.allclose(ssim, ref_ssim, rtol=SSIM_RTOL, atol=0)


def test_noalloc_rejects_textures_beyond_its_scratch(native):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    assert native.nebc7_init_device(1) == 0
    st = _settings(1, 9, 1, 0, 0)
    small = torch.zeros(4096, dtype=torch.uint8, device=dev)
    # 1024 x 1028 pixels = 65792 blocks: one block row past the capacity;
    # the call returns before any device work, so the small buffers are never read
    assert 1024 * 1028 // 16 > MAX_BLOCKS
    rc = native.nebc7_encode_device_noalloc(small.data_ptr(), small.data_ptr(), None, 1024 * 4, 1024, 1028,
                                            ctypes.byref(st), None, None)
    assert rc == 6
    assert native.nebc7_last_error() == 6
