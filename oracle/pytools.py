"""Numpy restatements of the reference driver's /bad and /map steps (test
infrastructure: the oracle for the device kernels of these steps; nothing
in the product imports it).

* bad_blocks: src/Worker.cpp:309-451 (ShowBadBlocks, DetectGlitches) with
  the thresholds of src/Bc7Tables.cpp:831-842.
* partition_map: src/Bc7Compress.cpp:131-265 (VisualizePartitionsGRB).
"""

from __future__ import annotations

import numpy as np


def bad_blocks(src: np.ndarray, dec: np.ndarray, mask: np.ndarray | None, linear: bool) -> np.ndarray:
    """src, dec: uint8[h, w, 4] BGRA (padded); mask: uint8[h, w, 4] bytes A, G, R, B or None."""
    h, w = src.shape[:2]
    d = np.abs(src.astype(np.int16) - dec.astype(np.int16)).astype(np.uint8)   # B, G, R, A
    m = np.full_like(src, 255) if mask is None else mask
    # the reference compares in A, G, R, B order against its per-channel steps
    dm = np.stack([d[..., 3] & m[..., 0], d[..., 1] & m[..., 1], d[..., 2] & m[..., 2], d[..., 0] & m[..., 3]], -1)
    thr = np.array([16, 16, 16, 16] if linear else [16, 12, 16, 20], np.int16)
    pix_bad = (dm.astype(np.int16) >= thr).any(-1)
    blk_bad = pix_bad.reshape(h // 4, 4, w // 4, 4).any(axis=(1, 3))
    out = np.zeros_like(src)
    sel = np.repeat(np.repeat(blk_bad, 4, 0), 4, 1)
    out[sel] = src[sel]
    return out


def _visualize(d0: int, d1: int) -> tuple[int, int]:
    m64 = (1 << 64) - 1
    if d0 & 0xF:
        if d0 & 3:
            if d0 & 1:
                return (d0 & 0x1F) | (0xF << 29) | (0xF << 13), 0xF << 5
            return (d0 & 0xFF) | (0x3F << 32) | (0x3F << 20), 0
        if d0 & 4:
            return (d0 & 0x1FF) | (0x1F << 39) | (0x1F << 19), 0x1F << 25
        return (d0 & 0x3FF) | (0x7F << 38) | (0x7F << 24), 0
    if d0 & 0xF0:
        if d0 & 0x30:
            if d0 & 0x10:
                return (d0 & 0x1F) | (0x1F << 18) | (0x1F << 8) | (0x3F << 38), 0
            return (d0 & 0x3F) | (0x7F << 22) | (0x7F << 8) | (0xFF << 50), 0
        if d0 & 0x40:
            if d0 == 0x40 and d1 == 0:
                return d0, d1
            idx = ((d1 & ~0xF) & m64) + ((d1 & 0xF) >> 1)
            c = 0x50 if ((idx >> 2) ^ idx) & 0x3333333333333333 else 0x30
            return (d0 & 0x7F) | (c << 21) | (c << 7) | (c << 35) | (0x7F << 49), 0
        return (d0 & 0x3FFF) | (0x1F << 34) | (0x1F << 24), (0x1F << 10) | (0x1F << 20)
    return d0, d1


def partition_map(blocks: np.ndarray) -> np.ndarray:
    """blocks: uint8[n, 16] -> the visualisation blocks."""
    b = np.ascontiguousarray(blocks).view(np.uint64).reshape(-1, 2)
    out = np.empty_like(b)
    for k in range(len(b)):
        d0, d1 = _visualize(int(b[k, 0]), int(b[k, 1]))
        out[k, 0], out[k, 1] = d0, d1
    return out.view(np.uint8).reshape(-1, 16)
