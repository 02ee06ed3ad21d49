"""Serving: requests submitted while others run come back with the blocks
and sums a plain single-texture encode gives them, alone and in the mix
(GPU)."""

import ctypes
import threading

import numpy as np
import pytest

from nebc7_gb300 import synth

pytestmark = pytest.mark.gpu

PRESETS = {"draft": (1, 9, 1, 0, 0, 0), "default": (1, 9, 1, 1, 0, 0), "precise": (0, 0, 1, 1, 0, 0),
           "m6i2": (1, 9, 2, 0, 0, 0), "slow": (1, 9, 1, 1, 1, 0)}


def _requests(n, seed):
    from nebc7_gb300.api import outline_mask, pad_texture
    names = list(PRESETS)
    out = []
    for i, d in enumerate(synth.batch_textures(n, seed, 4, 128)):
        img = pad_texture(synth.image_for(d["kind"], d["w"], d["h"], d["seed"]))
        mask = outline_mask(img, 1) if d["alpha"] else None
        out.append((img, mask, names[i % len(names)]))
    return out


def _plain(native, img, mask, preset):
    from nebc7_gb300._native import Settings
    h, w = img.shape[:2]
    dst = np.zeros(((h // 4) * (w // 4), 16), np.uint8)
    errs = np.zeros(2, np.int64)
    ssim = np.zeros(2, np.float64)
    st = Settings(*PRESETS[preset])
    assert native.nebc7_encode_host(dst.ctypes.data, img.ctypes.data, mask.ctypes.data if mask is not None else None,
                                    w * 4, w, h, ctypes.byref(st), errs.ctypes.data, ssim.ctypes.data) == 0
    return dst, errs, ssim


def test_server_results_match_plain_encodes_alone_and_mixed(native):
    from nebc7_gb300 import Server
    from nebc7_gb300._native import Settings
    reqs = _requests(25, 5)
    want = [_plain(native, *r) for r in reqs]
    # a small arena forces queueing behind the memory budget; two streams overlap batches
    srv = Server(hbm_budget=3 << 20, max_batch=4, streams=2)
    outs, tickets = [], []
    for img, mask, preset in reqs:
        h, w = img.shape[:2]
        dst = np.full(((h // 4) * (w // 4), 16), 0xAA, np.uint8)   # outputs start from scratch regardless
        outs.append(dst)
        tickets.append(srv.submit(img, mask, dst, Settings(*PRESETS[preset])))
    infos = [srv.wait(t) for t in tickets]
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["peak_bytes"] <= 3 << 20
    for i, (dst, info) in enumerate(zip(outs, infos)):
        assert np.array_equal(dst, want[i][0]), f"request {i} ({reqs[i][2]})"
        assert info["errs"] == want[i][1].tolist()
        assert info["ssim"] == want[i][2].tolist()
        assert info["latency_ms"] >= info["queue_ms"] >= 0
    # each request alone through the same server
    for i in (0, 3, 7):
        img, mask, preset = reqs[i]
        h, w = img.shape[:2]
        dst = np.zeros(((h // 4) * (w // 4), 16), np.uint8)
        info = srv.wait(srv.submit(img, mask, dst, Settings(*PRESETS[preset])))
        assert np.array_equal(dst, outs[i]) and info["errs"] == infos[i]["errs"]
    srv.close()


def test_server_accepts_submissions_from_several_threads(native):
    from nebc7_gb300 import Server
    from nebc7_gb300._native import Settings
    reqs = _requests(12, 9)
    want = [_plain(native, *r) for r in reqs]
    srv = Server(hbm_budget=64 << 20, max_batch=8, streams=3)
    outs = [np.zeros(((r[0].shape[0] // 4) * (r[0].shape[1] // 4), 16), np.uint8) for r in reqs]
    tickets = [None] * len(reqs)

    def submit(idx):
        for i in idx:
            img, mask, preset = reqs[i]
            tickets[i] = srv.submit(img, mask, outs[i], Settings(*PRESETS[preset]))

    th = [threading.Thread(target=submit, args=(range(k, len(reqs), 2),)) for k in (0, 1)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i, t in enumerate(tickets):
        srv.wait(t)
        assert np.array_equal(outs[i], want[i][0])
    srv.close()


def test_server_rejects_requests_beyond_its_budget(native):
    from nebc7_gb300 import NativeError, Server
    from nebc7_gb300._native import Settings
    srv = Server(hbm_budget=1 << 16, max_batch=2, streams=1)
    img = np.zeros((256, 256, 4), np.uint8)
    dst = np.zeros((64 * 64, 16), np.uint8)
    with pytest.raises(NativeError) as e:
        srv.submit(img, None, dst, Settings(*PRESETS["draft"]))
    assert e.value.code == 6
    srv.close()


def test_server_admits_requests_while_others_run(native):
    """Continuous batching: requests that arrive while a long launch is on
    the device start on another slot and come back before it ends, with the
    blocks a plain encode gives them."""
    import time
    from nebc7_gb300 import Server
    from nebc7_gb300._native import Settings
    big = synth.image_for("photo_like", 1024, 512, 21)
    small = _requests(6, 22)
    srv = Server(hbm_budget=256 << 20, max_batch=4, streams=2)
    big_out = np.zeros(((512 // 4) * (1024 // 4), 16), np.uint8)
    t_big = srv.submit(big, None, big_out, Settings(*PRESETS["precise"]))
    time.sleep(0.005)
    outs, tickets = [], []
    for img, mask, preset in small:
        h, w = img.shape[:2]
        outs.append(np.zeros(((h // 4) * (w // 4), 16), np.uint8))
        tickets.append(srv.submit(img, mask, outs[-1], Settings(*PRESETS[preset])))
    infos = [srv.wait(t) for t in tickets]
    b = srv.wait(t_big)
    srv.close()
    joined = [s for s in infos
              if s["submit_at_ms"] > b["launch_at_ms"] and s["launch_at_ms"] < b["done_at_ms"]
              and s["done_at_ms"] < b["done_at_ms"] and s["slot"] != b["slot"] and s["launch"] != b["launch"]]
    assert joined, (b, infos)
    assert np.array_equal(big_out, _plain(native, big, None, "precise")[0])
    for i, (img, mask, preset) in enumerate(small):
        assert np.array_equal(outs[i], _plain(native, img, mask, preset)[0])
