"""Python host side of the encoder, shaped like the reference's interfaces.

* ``Bc7Core`` mirrors the reference's ``IBc7Core`` vtable (reference
  src/Bc7Core.h:316-322): ``init_tables`` (pInitTables), ``compress`` /
  ``decompress`` (pCompress / pDecompress over independent 4x4 cells) and
  ``weight_alpha`` / ``weight_color``.  The preset (kDenoise, kDenoiseStep),
  a compile-time constant in the reference (src/Bc7Mode.h:10-13), is a
  constructor argument here.
* ``process_texture`` mirrors ``ProcessTexture`` (src/Worker.h:6) on a padded
  texture.
* ``encode_image`` mirrors the CLI driver (src/Bc7Compress.cpp:267): CLI
  flags, padding to multiples of 4, the alpha outline mask, the encode, and
  the qMSE / qPSNR / wSSIM report.
* ``encode_device`` works on resident device buffers (torch CUDA tensors or raw
  pointers) with a CUDA stream.

Everything runs on the GPU through the C ABI; nothing here computes blocks.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _native
from ._native import NativeError, Settings, check


@dataclass(frozen=True)
class Preset:
    """The reference's kDenoise / kDenoiseStep pair (src/Bc7Mode.h:10-13)."""

    denoise: int = 1
    step: int = 9


DEFAULT = Preset(1, 9)
PRECISE = Preset(0, 0)


def _settings(preset: Preset, draft: bool, normal: bool, slow: bool, linear: bool) -> Settings:
    return Settings(int(preset.denoise), int(preset.step), int(draft), int(normal), int(slow), int(linear))


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


@dataclass
class EncodeStats:
    """Error and SSIM sums as the reference's block kernel accumulates them
    (src/Bc7Core.cpp:1980-1984)."""

    err_alpha: int
    err_color: int
    ssim_alpha: float
    ssim_color: float


class Bc7Core:
    """The IBc7Core block API over the GPU encoder."""

    def __init__(self, preset: Preset = DEFAULT):
        self.preset = preset
        self._lib = _native.load()
        self._flags = (True, True, False, False)

    def init_tables(self, do_draft: bool = True, do_normal: bool = True, do_slow: bool = False,
                    linear_data: bool = False) -> None:
        """pInitTables (src/Bc7Core.cpp:1877): flags, weights and resident tables."""
        draft = 2 if do_draft == 2 else bool(do_draft)   # 2: the Mode6Index2 fast run
        self._flags = (draft, bool(do_normal), bool(do_slow), bool(linear_data))
        check(self._lib.nebc7_init_device(int(self.preset.denoise)), "init tables")

    def weight_alpha(self) -> int:
        return 1 if self._flags[3] else 1000

    def weight_color(self) -> int:
        return 3 if self._flags[3] else 715 + 213 + 72

    def settings(self) -> Settings:
        return _settings(self.preset, *self._flags)

    def compress(self, cells: np.ndarray, masks: np.ndarray, blocks: np.ndarray) -> EncodeStats:
        """pCompress over n cells: cells / masks uint8[n, 64], blocks uint8[n, 16]
        (starting blocks in, results out)."""
        cells = np.ascontiguousarray(cells, dtype=np.uint8)
        masks = np.ascontiguousarray(masks, dtype=np.uint8)
        if blocks.dtype != np.uint8 or not blocks.flags.c_contiguous:
            raise ValueError("blocks must be a C-contiguous uint8 array")
        n = blocks.shape[0]
        if cells.shape != (n, 64) or masks.shape != (n, 64) or blocks.shape != (n, 16):
            raise ValueError("expected cells/masks [n, 64] and blocks [n, 16]")
        err = np.zeros(2, np.int64)
        ssim = np.zeros(2, np.float64)
        s = self.settings()
        check(self._lib.nebc7_encode_blocks_host(_ptr(cells), _ptr(masks), _ptr(blocks), n, ctypes.byref(s),
                                                 _ptr(err), _ptr(ssim)), "compress")
        return EncodeStats(int(err[0]), int(err[1]), float(ssim[0]), float(ssim[1]))

    def decompress(self, blocks: np.ndarray) -> np.ndarray:
        """pDecompress: uint8[n, 16] blocks -> uint8[n, 64] BGRA cells."""
        blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
        out = np.zeros((blocks.shape[0], 64), np.uint8)
        check(self._lib.nebc7_decode_blocks_host(_ptr(blocks), _ptr(out), blocks.shape[0]), "decompress")
        return out

    def process_texture(self, dst: np.ndarray, src_bgra: np.ndarray, mask_agrb: np.ndarray | None,
                        width: int, height: int, stride: int | None = None) -> EncodeStats:
        """ProcessTexture (src/Worker.h:6) with the compress kernel on a padded
        texture held in host arrays."""
        stride = width * 4 if stride is None else stride
        src_bgra = np.ascontiguousarray(src_bgra, dtype=np.uint8)
        mp = None
        if mask_agrb is not None:
            mask_agrb = np.ascontiguousarray(mask_agrb, dtype=np.uint8)
            mp = _ptr(mask_agrb)
        err = np.zeros(2, np.int64)
        ssim = np.zeros(2, np.float64)
        s = self.settings()
        check(self._lib.nebc7_encode_host(_ptr(dst), _ptr(src_bgra), mp, stride, width, height, ctypes.byref(s),
                                          _ptr(err), _ptr(ssim)), "process_texture")
        return EncodeStats(int(err[0]), int(err[1]), float(ssim[0]), float(ssim[1]))


def padded_size(w: int, h: int) -> tuple[int, int]:
    """src/Bc7Compress.cpp:397-398: at least 4, rounded up to a multiple of 4."""
    return (max(4, w) + 3) & ~3, (max(4, h) + 3) & ~3


def pad_texture(img_bgra: np.ndarray) -> np.ndarray:
    """Edge replication to the padded size (src/Bc7Compress.cpp:411-426)."""
    h, w = img_bgra.shape[:2]
    pw, ph = padded_size(w, h)
    out = np.empty((ph, pw, 4), np.uint8)
    out[:h, :w] = img_bgra
    out[:h, w:] = img_bgra[:, w - 1:w]
    out[h:] = out[h - 1:h]
    return out


def outline_mask(padded_bgra: np.ndarray, radius: int) -> np.ndarray:
    """Alpha mask with an outline (src/Bc7Compress.cpp:33-105): colour is
    visible where any pixel of the (2r+1)^2 neighbourhood has non-zero alpha;
    alpha is always visible.  Bytes A,G,R,B per pixel."""
    h, w = padded_bgra.shape[:2]
    on = (padded_bgra[:, :, 3] != 0).astype(np.int32)
    pad = np.pad(on, radius)
    c = pad.cumsum(0).cumsum(1)
    c = np.pad(c, ((1, 0), (1, 0)))
    k = 2 * radius + 1
    box = c[k:k + h, k:k + w] - c[0:h, k:k + w] - c[k:k + h, 0:w] + c[0:h, 0:w]
    mask = np.empty((h, w, 4), np.uint8)
    mask[:, :, 0] = 0xFF
    v = np.where(box > 0, 0xFF, 0).astype(np.uint8)
    mask[:, :, 1] = v
    mask[:, :, 2] = v
    mask[:, :, 3] = v
    return mask


def parse_flags(flags: str) -> dict:
    """CLI switches (src/Bc7Compress.cpp:269-363) that affect the encode."""
    o = dict(draft=True, normal=True, slow=False, mask=True, radius=1, linear=False)
    for f in flags.split():
        if f == "/draft":
            o.update(draft=True, normal=False, slow=False)
        elif f == "/slow":
            o.update(draft=True, normal=True, slow=True)
        elif f == "/nomask":
            o["mask"] = False
        elif f == "/retina":
            o["radius"] = 2
        elif f == "/data":
            o.update(mask=False, linear=True)
        elif f == "/compare":
            o.update(draft=False, normal=False, slow=False)
        elif f == "/m6i2":
            # the "Mode6Index2 fast" run: the draft chain reduced to its
            # Mode6Index2 pass (no counterpart switch in the reference CLI)
            o.update(draft=2, normal=False, slow=False)
        elif f == "/noflip":
            pass
        else:
            raise ValueError(f"unsupported flag {f!r}")
    return o


@dataclass
class EncodedImage:
    blocks: np.ndarray       # uint8[padded_h // 4 * padded_w // 4, 16]
    width: int               # padded texture size
    height: int
    stats: EncodeStats

    def report(self, weight_alpha: int, weight_color: int) -> dict:
        """qMSE / qPSNR / SSIM as the CLI prints them (src/Bc7Compress.cpp:490-518)."""
        px = self.width * self.height
        out = {}
        if self.stats.err_alpha > 0:
            out["A"] = dict(qMSE=self.stats.err_alpha / weight_alpha / px,
                            qPSNR=10.0 * math.log(255.0 * 255.0 * weight_alpha * px / self.stats.err_alpha) / math.log(10.0),
                            SSIM_4x4=self.stats.ssim_alpha * 16.0 / px)
        if self.stats.err_color > 0:
            out["RGB"] = dict(qMSE=self.stats.err_color / weight_color / px,
                              qPSNR=10.0 * math.log(255.0 * 255.0 * weight_color * px / self.stats.err_color) / math.log(10.0),
                              wSSIM_4x4=self.stats.ssim_color * 16.0 / px)
        return out


def encode_image(img_bgra: np.ndarray, flags: str = "", preset: Preset = DEFAULT,
                 start: np.ndarray | None = None) -> EncodedImage:
    """The CLI's encode path on an in-memory BGRA image (top-down rows)."""
    o = parse_flags(flags)
    padded = pad_texture(np.ascontiguousarray(img_bgra, dtype=np.uint8))
    ph, pw = padded.shape[:2]
    mask = outline_mask(padded, o["radius"]) if o["mask"] else None
    core = Bc7Core(preset)
    core.init_tables(o["draft"], o["normal"], o["slow"], o["linear"])
    blocks = np.zeros(((ph // 4) * (pw // 4), 16), np.uint8) if start is None else np.array(start, np.uint8)
    stats = core.process_texture(blocks, padded, mask, pw, ph)
    return EncodedImage(blocks, pw, ph, stats)


def set_pca(on: bool) -> None:
    """OPTION_PCA for the encodes, batches and servers created afterwards
    (off by default, as in the reference's build; PCA-on outputs are not
    pinned to the reference, whose axis comes from the absent Eigen)."""
    check(_native.load().nebc7_set_pca(int(bool(on))), "set_pca")


def encode_device(dst_ptr: int, bgra_ptr: int, mask_ptr: int | None, stride: int, width: int, height: int,
                  preset: Preset = DEFAULT, draft: bool = True, normal: bool = True, slow: bool = False,
                  linear: bool = False, stream: int = 0, want_stats: bool = False) -> EncodeStats | None:
    """Encodes device-resident buffers (raw CUDA pointers) on `stream`."""
    lib = _native.load()
    s = _settings(preset, draft, normal, slow, linear)
    if want_stats:
        err = np.zeros(2, np.int64)
        ssim = np.zeros(2, np.float64)
        check(lib.nebc7_encode_device(dst_ptr, bgra_ptr, mask_ptr, stride, width, height, ctypes.byref(s),
                                      _ptr(err), _ptr(ssim), stream), "encode_device")
        return EncodeStats(int(err[0]), int(err[1]), float(ssim[0]), float(ssim[1]))
    check(lib.nebc7_encode_device(dst_ptr, bgra_ptr, mask_ptr, stride, width, height, ctypes.byref(s),
                                  None, None, stream), "encode_device")
    return None


@dataclass
class BatchTexture:
    """One texture of a Batch: raw CUDA device pointers and its own preset."""

    dst: int
    bgra: int
    mask: int | None
    stride: int
    width: int
    height: int
    settings: Settings


def plan_key(textures: list[BatchTexture], device: str) -> str:
    """The (preset mix, GPU) a tuned batch plan is kept for: the device name
    and, per preset, its blocks rounded down to a power of two, so that
    batches of the same mix and about the same size share a plan."""
    mix: dict[tuple, int] = {}
    for t in textures:
        s = t.settings
        k = (s.denoise, s.denoiseStep, s.doDraft, s.doNormal, s.doSlow, s.linearData)
        mix[k] = mix.get(k, 0) + (t.width // 4) * (t.height // 4)
    parts = [f"{'-'.join(map(str, k))}:{1 << max(0, v.bit_length() - 1)}" for k, v in sorted(mix.items())]
    return device + "|" + ",".join(parts)


class PlanStore:
    """Tuned batch plans in a JSON file, one per plan_key, so that a batch of
    a known mix on a known GPU starts from its plan instead of tuning."""

    def __init__(self, path):
        import pathlib
        self.path = pathlib.Path(path)

    def _read(self) -> dict:
        import json
        return json.loads(self.path.read_text()) if self.path.exists() else {}

    def get(self, key: str) -> dict | None:
        return self._read().get(key)

    def put(self, key: str, plan: dict) -> None:
        import json
        import os
        plans = self._read()
        plans[key] = {"schedule": plan["schedule"], "staged": bool(plan["staged"]), "ctas_per_sm": int(plan["ctas_per_sm"])}
        tmp = self.path.with_suffix(self.path.suffix + ".tmp")
        tmp.write_text(json.dumps(plans, indent=1, sort_keys=True))
        os.replace(tmp, self.path)


class Batch:
    """Many textures of any sizes and presets encoded by one plan: a
    persistent launch over a global block queue (or one per preset group on
    concurrent streams), replayed as a CUDA graph.  Device buffers stay the
    caller's and must outlive the Batch."""

    MIXED, GROUPED = 0, 1

    def __init__(self, textures: list[BatchTexture], from_scratch: bool = False):
        self._textures = list(textures)
        self._lib = _native.load()
        arr = (_native.Texture * len(textures))()
        for i, t in enumerate(textures):
            arr[i].d_dst = t.dst
            arr[i].d_bgra = t.bgra
            arr[i].d_mask = t.mask
            arr[i].stride = t.stride
            arr[i].w = t.width
            arr[i].h = t.height
            arr[i].settings = t.settings
        self._n = len(textures)
        self._h = ctypes.c_void_p()
        check(self._lib.nebc7_batch_create(ctypes.cast(arr, ctypes.c_void_p), self._n,
                                           _native.BATCH_FROM_SCRATCH if from_scratch else 0,
                                           ctypes.byref(self._h)), "batch_create")

    def tune(self, trials: int = 2) -> tuple[float, float]:
        """Searches the plan's knobs (schedule, staged form, CTAs per SM),
        timing each candidate `trials` times as a CUDA graph, and keeps the
        fastest (trials() lists them); returns the best ms of the mixed and
        the grouped schedule."""
        ms = (ctypes.c_float * 2)()
        check(self._lib.nebc7_batch_tune(self._h, trials, ctypes.cast(ms, ctypes.c_void_p)), "batch_tune")
        return float(ms[0]), float(ms[1])

    def set_schedule(self, which: int) -> None:
        check(self._lib.nebc7_batch_set_schedule(self._h, which), "batch_set_schedule")

    def plan(self) -> dict:
        """The plan's knobs: schedule, staged form, CTAs per SM (0: occupancy)."""
        s, st, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self._lib.nebc7_batch_plan(self._h, ctypes.byref(s), ctypes.byref(st), ctypes.byref(c)), "batch_plan")
        return {"schedule": ("mixed", "grouped")[s.value], "staged": bool(st.value), "ctas_per_sm": c.value}

    def set_plan(self, schedule: int, staged: bool, ctas_per_sm: int = 0) -> None:
        check(self._lib.nebc7_batch_set_plan(self._h, schedule, int(staged), ctas_per_sm), "batch_set_plan")

    def tune_cached(self, store: PlanStore, device: str, trials: int = 2) -> tuple[dict, bool]:
        """The plan kept in `store` for this batch's mix on `device` if there
        is one, else tune() and keep its choice; returns the plan and whether
        it was tuned now."""
        key = plan_key(self._textures, device)
        plan = store.get(key)
        if plan is not None:
            self.set_plan(("mixed", "grouped").index(plan["schedule"]), plan["staged"], plan["ctas_per_sm"])
            return self.plan(), False
        self.tune(trials)
        plan = self.plan()
        store.put(key, plan)
        return plan, True

    def trials(self) -> list[dict]:
        """The plans the last tune timed, in order, with their best ms."""
        n = self._lib.nebc7_batch_trials(self._h, None, None, None, None, 0)
        if n <= 0:
            return []
        s, st, c = (ctypes.c_int * n)(), (ctypes.c_int * n)(), (ctypes.c_int * n)()
        ms = (ctypes.c_float * n)()
        self._lib.nebc7_batch_trials(self._h, s, st, c, ms, n)
        return [{"schedule": ("mixed", "grouped")[s[i]], "staged": bool(st[i]), "ctas_per_sm": c[i],
                 "ms": float(ms[i])} for i in range(n)]

    def launch(self, stream: int = 0) -> None:
        check(self._lib.nebc7_batch_launch(self._h, stream), "batch_launch")

    def sums(self, stream: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """Per-texture (errAlpha, errColor) and (ssimAlpha, ssimColor) of the last launch."""
        errs = np.zeros((self._n, 2), np.int64)
        ssim = np.zeros((self._n, 2), np.float64)
        check(self._lib.nebc7_batch_sums(self._h, stream, _ptr(errs), _ptr(ssim)), "batch_sums")
        return errs, ssim

    def info(self) -> dict:
        sched, launches, blocks = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self._lib.nebc7_batch_info(self._h, ctypes.byref(sched), ctypes.byref(launches),
                                         ctypes.byref(blocks)), "batch_info")
        return {"schedule": ("mixed", "grouped")[sched.value], "launches": launches.value, "blocks": blocks.value}

    def close(self) -> None:
        if self._h:
            self._lib.nebc7_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


KTX_HEADER_BYTES = 96


def ktx_header(width: int, height: int, flip: bool = False) -> bytes:
    """The KTX 1.1 header the reference's driver writes for a BC7 image."""
    out = (ctypes.c_uint8 * KTX_HEADER_BYTES)()
    check(_native.load().nebc7_ktx_header(width, height, int(flip), ctypes.cast(out, ctypes.c_void_p)), "ktx_header")
    return bytes(out)


def write_ktx(path: str, blocks: np.ndarray, width: int, height: int, flip: bool = False) -> None:
    """Saves blocks (uint8[n, 16] of the padded texture) as a .ktx file."""
    pw, ph = padded_size(width, height)
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    if blocks.size != pw * ph:
        raise ValueError(f"{blocks.size} bytes of blocks for a {pw}x{ph} texture")
    with open(path, "wb") as f:
        f.write(ktx_header(width, height, flip))
        f.write(blocks.tobytes())


def read_ktx(path: str) -> tuple[np.ndarray, int, int, bool]:
    """Loads a .ktx written by write_ktx (or the reference): (blocks, width,
    height, flip).  The blocks can seed an incremental re-encode (`start`)."""
    data = open(path, "rb").read()
    head = np.frombuffer(data[:KTX_HEADER_BYTES], np.uint32)
    if len(data) < KTX_HEADER_BYTES or head[0] != 0x58544BAB or head[7] != 0x8E8C:
        raise ValueError(f"{path}: not a BC7 KTX file")
    width, height = int(head[9]), int(head[10])
    size = int(head[23])
    flip = int(head[22]) == 0x00753D
    blocks = np.frombuffer(data[KTX_HEADER_BYTES:KTX_HEADER_BYTES + size], np.uint8).reshape(-1, 16).copy()
    return blocks, width, height, flip


class Server:
    """Request loop on the current device: textures are submitted as they
    arrive (host buffers) and come back encoded; see nebc7_server_create."""

    def __init__(self, hbm_budget: int = 64 << 30, max_batch: int = 64, streams: int = 4):
        self._lib = _native.load()
        cfg = _native.ServerConfig(hbm_budget, max_batch, streams)
        self._h = ctypes.c_void_p()
        check(self._lib.nebc7_server_create(ctypes.byref(cfg), ctypes.byref(self._h)), "server_create")
        self._keep = {}

    def submit(self, bgra: np.ndarray, mask: np.ndarray | None, dst: np.ndarray, settings: Settings) -> int:
        """Queues one padded texture; `dst` (uint8[w*h/16, 16]) receives the blocks."""
        h, w = bgra.shape[:2]
        ticket = ctypes.c_int64()
        check(self._lib.nebc7_server_submit(self._h, _ptr(bgra), _ptr(mask) if mask is not None else None, w * 4, w, h,
                                            ctypes.byref(settings), _ptr(dst), ctypes.byref(ticket)), "server_submit")
        self._keep[ticket.value] = (bgra, mask, dst)
        return ticket.value

    def wait(self, ticket: int, timeout: float = -1.0) -> dict:
        info = _native.RequestInfo()
        rc = self._lib.nebc7_server_wait(self._h, ticket, timeout, ctypes.byref(info))
        check(rc, "server_wait")
        self._keep.pop(ticket, None)
        return {"queue_ms": info.queue_ms, "latency_ms": info.latency_ms, "errs": [info.errs[0], info.errs[1]],
                "ssim": [info.ssim[0], info.ssim[1]], "submit_at_ms": info.submit_at_ms,
                "launch_at_ms": info.launch_at_ms, "done_at_ms": info.done_at_ms, "slot": info.slot,
                "launch": info.launch}

    def stats(self) -> dict:
        c = _native.ServerCounters()
        check(self._lib.nebc7_server_stats(self._h, ctypes.byref(c)), "server_stats")
        return {k: getattr(c, k) for k, _ in c._fields_}

    def close(self) -> None:
        if self._h:
            self._lib.nebc7_server_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = [
    "Bc7Core", "Preset", "DEFAULT", "PRECISE", "EncodeStats", "EncodedImage", "NativeError",
    "encode_image", "encode_device", "set_pca", "pad_texture", "outline_mask", "padded_size", "parse_flags",
    "Batch", "BatchTexture", "Server", "ktx_header", "write_ktx", "read_ktx",
]
