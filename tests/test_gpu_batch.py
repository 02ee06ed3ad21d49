"""Batches: one plan over textures of mixed sizes and presets, replayed as a
CUDA graph, gives for every texture the blocks and sums of a plain
single-texture encode (GPU)."""

import ctypes

import numpy as np
import pytest

from nebc7_gb300 import synth

pytestmark = pytest.mark.gpu

PRESETS = {"draft": (1, 9, 1, 0, 0, 0), "default": (1, 9, 1, 1, 0, 0), "precise": (0, 0, 1, 1, 0, 0),
           "slow": (1, 9, 1, 1, 1, 0), "data": (1, 9, 1, 1, 0, 1)}


def _textures(torch, n, seed, lo, hi, presets=None):
    from nebc7_gb300.api import outline_mask, pad_texture
    dev = torch.device("cuda", 0)
    out = []
    for i, d in enumerate(synth.batch_textures(n, seed, lo, hi)):
        img = pad_texture(synth.image_for(d["kind"], d["w"], d["h"], d["seed"]))
        mask = outline_mask(img, 1) if d["alpha"] else None
        h, w = img.shape[:2]
        preset = presets[i % len(presets)] if presets else d["preset"]
        out.append({"w": w, "h": h, "img": torch.from_numpy(img).to(dev),
                    "mask": torch.from_numpy(mask).to(dev) if mask is not None else None,
                    "dst": torch.zeros((h // 4) * (w // 4) * 16, dtype=torch.uint8, device=dev),
                    "preset": preset})
    return out


def _plain(native, torch, t):
    from nebc7_gb300._native import Settings
    st = Settings(*PRESETS[t["preset"]])
    dst = torch.zeros_like(t["dst"])
    errs = np.zeros(2, np.int64)
    ssim = np.zeros(2, np.float64)
    rc = native.nebc7_encode_device(dst.data_ptr(), t["img"].data_ptr(),
                                    t["mask"].data_ptr() if t["mask"] is not None else None, t["w"] * 4, t["w"], t["h"],
                                    ctypes.byref(st), errs.ctypes.data, ssim.ctypes.data, None)
    assert rc == 0
    return dst.cpu().numpy(), errs, ssim


def _batch(texs, from_scratch=True):
    from nebc7_gb300 import Batch, BatchTexture
    from nebc7_gb300._native import Settings
    return Batch([BatchTexture(t["dst"].data_ptr(), t["img"].data_ptr(),
                               t["mask"].data_ptr() if t["mask"] is not None else None, t["w"] * 4, t["w"], t["h"],
                               Settings(*PRESETS[t["preset"]])) for t in texs], from_scratch=from_scratch)


@pytest.mark.parametrize("schedule", [0, 1])
def test_batch_matches_plain_launches(native, schedule):
    torch = pytest.importorskip("torch")
    texs = _textures(torch, 20, 31, 4, 128, ["draft", "default", "precise", "slow", "data"])
    want = [_plain(native, torch, t) for t in texs]
    b = _batch(texs)
    b.set_schedule(schedule)
    for rep in range(2):   # graph replays
        b.launch()
        errs, ssim = b.sums()
        for i, t in enumerate(texs):
            blocks, e, q = want[i]
            assert np.array_equal(t["dst"].cpu().numpy(), blocks), f"texture {i} ({t['preset']}, {t['w']}x{t['h']})"
            assert errs[i].tolist() == e.tolist()
            assert np.array_equal(ssim[i], q)
    b.close()


@pytest.mark.parametrize("plan", [(0, 0, 0), (0, 1, 1), (1, 0, 2), (1, 1, 3)])
def test_every_plan_gives_the_plain_blocks(native, plan):
    """The tuner's knobs (schedule, staged form, CTAs per SM) change how the
    blocks are scheduled, never what they are."""
    torch = pytest.importorskip("torch")
    texs = _textures(torch, 15, 53, 4, 128, ["precise", "default", "slow", "draft", "data"])
    want = [_plain(native, torch, t) for t in texs]
    b = _batch(texs)
    b.set_plan(*plan)
    assert b.plan() == {"schedule": ("mixed", "grouped")[plan[0]], "staged": bool(plan[1]), "ctas_per_sm": plan[2]}
    b.launch()
    errs, ssim = b.sums()
    for i, t in enumerate(texs):
        blocks, e, q = want[i]
        assert np.array_equal(t["dst"].cpu().numpy(), blocks), f"texture {i} ({t['preset']})"
        assert errs[i].tolist() == e.tolist()
        assert np.array_equal(ssim[i], q)
    b.close()


def test_batch_tune_keeps_outputs_and_starting_blocks(native):
    torch = pytest.importorskip("torch")
    texs = _textures(torch, 12, 47, 16, 256)
    want = [_plain(native, torch, t) for t in texs]
    starts = [t["dst"].clone() for t in texs]
    b = _batch(texs, from_scratch=False)
    ms = b.tune(1)
    assert min(ms) > 0
    for t, s in zip(texs, starts):      # tuning restores the starting blocks
        assert torch.equal(t["dst"], s)
    b.launch()
    errs, _ = b.sums()
    for i, t in enumerate(texs):
        assert np.array_equal(t["dst"].cpu().numpy(), want[i][0])
        assert errs[i].tolist() == want[i][1].tolist()
    info = b.info()
    assert info["blocks"] == sum((t["w"] // 4) * (t["h"] // 4) for t in texs)
    trials = b.trials()
    assert len(trials) >= 2 and all(t["ms"] > 0 for t in trials)
    p = b.plan()
    assert min(t["ms"] for t in trials) == min(t["ms"] for t in trials
                                               if (t["schedule"], t["staged"], t["ctas_per_sm"]) ==
                                               (p["schedule"], p["staged"], p["ctas_per_sm"]))
    b.close()


def test_batch_rejects_bad_textures(native):
    from nebc7_gb300._native import Settings, Texture
    arr = (Texture * 1)()
    arr[0].w, arr[0].h, arr[0].stride = 6, 4, 24
    arr[0].settings = Settings(1, 9, 1, 0, 0, 0)
    h = ctypes.c_void_p()
    assert native.nebc7_batch_create(ctypes.cast(arr, ctypes.c_void_p), 1, 0, ctypes.byref(h)) == 1
    assert native.nebc7_batch_create(None, 0, 0, ctypes.byref(h)) == 1
