"""Seeded synthetic RGBA8 images for the encoder's workloads.

The reference is benchmarked on photographs that are not available here, so
every workload uses images produced by this module.  All arithmetic is
integer (numpy uint64 / int64) so an image is bit-identical on any platform
and numpy version: the random stream is SplitMix64, value noise is bilinear
interpolation in 16.16 fixed point, and shapes are rasterised with exact
integer edge functions.

Images are returned as ``uint8[h, w, 4]`` in **BGRA** byte order, the order the
block API reads (reference src/Bc7Core.cpp:1866 ConvertBgraToAgrb).

Workloads (sizes and value distributions follow the encoder's published
benchmark set-ups; the images themselves are synthetic):

* ``gradient_noise(w, h, seed)``: opaque; bilinear gradient between four
  random corner colours + 8x8-cell value noise (amplitude 40) + uniform
  integer noise in [-3, 3].
* ``photo_like(w, h, seed)``: opaque; four octaves of value noise (cells
  64/32/16/8, amplitudes 96/48/24/12, channels correlated with rho = 0.8),
  200 hard-edged random polygons, +-1 uniform noise.
* ``alpha_blobs(w, h, seed)``: non-premultiplied RGBA; ~30 % alpha = 0 in
  blob-shaped regions with random RGB, ~15 % a smooth alpha ramp 1..254, the
  rest opaque; RGB as in ``gradient_noise``.
"""

from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


class SplitMix64:
    """Counter-based SplitMix64 stream (Steele et al. 2014), vectorised."""

    def __init__(self, seed: int):
        self._state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)

    def u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            idx = np.arange(1, n + 1, dtype=np.uint64)
            z = self._state + idx * np.uint64(0x9E3779B97F4A7C15)
            self._state = self._state + np.uint64(n) * np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        return z

    def below(self, bound: int, n: int) -> np.ndarray:
        """n integers uniform in [0, bound) (multiply-shift; bias < 2^-32)."""
        r = self.u64(n) >> np.uint64(32)
        return ((r * np.uint64(bound)) >> np.uint64(32)).astype(np.int64)

    def between(self, lo: int, hi: int, n: int) -> np.ndarray:
        """n integers uniform in [lo, hi]."""
        return lo + self.below(hi - lo + 1, n)


def _value_noise(rng: SplitMix64, w: int, h: int, cell: int, amplitude: int) -> np.ndarray:
    """Bilinear value noise in [-amplitude, amplitude], int64[h, w]."""
    gw = w // cell + 2
    gh = h // cell + 2
    lattice = rng.between(-amplitude, amplitude, gw * gh).reshape(gh, gw)
    ys = np.arange(h, dtype=np.int64)
    xs = np.arange(w, dtype=np.int64)
    y0 = ys // cell
    x0 = xs // cell
    fy = ((ys % cell) << 16) // cell  # 16.16 fractions
    fx = ((xs % cell) << 16) // cell
    a = lattice[y0][:, x0]
    b = lattice[y0][:, x0 + 1]
    c = lattice[y0 + 1][:, x0]
    d = lattice[y0 + 1][:, x0 + 1]
    one = np.int64(1 << 16)
    top = a * (one - fx)[None, :] + b * fx[None, :]
    bot = c * (one - fx)[None, :] + d * fx[None, :]
    v = top * (one - fy)[:, None] + bot * fy[:, None]
    # round half away from zero, exact in integers
    s = np.sign(v)
    return s * ((np.abs(v) + (np.int64(1) << 31)) >> 32)


def _gradient(rng: SplitMix64, w: int, h: int) -> np.ndarray:
    """Bilinear gradient between 4 random corner colours, int64[h, w, 3]."""
    corners = rng.between(0, 255, 12).reshape(4, 3)
    ys = np.arange(h, dtype=np.int64)
    xs = np.arange(w, dtype=np.int64)
    wx = (xs << 16) // max(w - 1, 1)
    wy = (ys << 16) // max(h - 1, 1)
    one = np.int64(1 << 16)
    out = np.empty((h, w, 3), dtype=np.int64)
    for ch in range(3):
        c00, c01, c10, c11 = corners[:, ch]
        top = c00 * (one - wx) + c01 * wx
        bot = c10 * (one - wx) + c11 * wx
        v = top[None, :] * (one - wy)[:, None] + bot[None, :] * wy[:, None]
        out[:, :, ch] = (v + (np.int64(1) << 31)) >> 32
    return out


def _to_bgra(rgb: np.ndarray, alpha: np.ndarray) -> np.ndarray:
    h, w = alpha.shape
    img = np.empty((h, w, 4), dtype=np.uint8)
    img[:, :, 0] = np.clip(rgb[:, :, 2], 0, 255)
    img[:, :, 1] = np.clip(rgb[:, :, 1], 0, 255)
    img[:, :, 2] = np.clip(rgb[:, :, 0], 0, 255)
    img[:, :, 3] = np.clip(alpha, 0, 255)
    return img


def _gradient_noise_rgb(rng: SplitMix64, w: int, h: int) -> np.ndarray:
    rgb = _gradient(rng, w, h)
    for ch in range(3):
        rgb[:, :, ch] += _value_noise(rng, w, h, 8, 40)
    rgb += rng.between(-3, 3, w * h * 3).reshape(h, w, 3)
    return rgb


def gradient_noise(w: int, h: int, seed: int = 0) -> np.ndarray:
    rng = SplitMix64(seed)
    rgb = _gradient_noise_rgb(rng, w, h)
    return _to_bgra(rgb, np.full((h, w), 255, dtype=np.int64))


def _fill_polygon(canvas: np.ndarray, pts: np.ndarray, colour: np.ndarray) -> None:
    """Fills a convex polygon (integer vertices, either winding) in place."""
    h, w = canvas.shape[:2]
    x0 = max(int(pts[:, 0].min()), 0)
    x1 = min(int(pts[:, 0].max()), w - 1)
    y0 = max(int(pts[:, 1].min()), 0)
    y1 = min(int(pts[:, 1].max()), h - 1)
    if x0 > x1 or y0 > y1:
        return
    ys, xs = np.mgrid[y0 : y1 + 1, x0 : x1 + 1].astype(np.int64)
    n = len(pts)
    pos = np.ones(ys.shape, dtype=bool)
    neg = np.ones(ys.shape, dtype=bool)
    for i in range(n):
        ax, ay = int(pts[i, 0]), int(pts[i, 1])
        bx, by = int(pts[(i + 1) % n, 0]), int(pts[(i + 1) % n, 1])
        e = (bx - ax) * (ys - ay) - (by - ay) * (xs - ax)
        pos &= e >= 0
        neg &= e <= 0
    inside = pos | neg
    sub = canvas[y0 : y1 + 1, x0 : x1 + 1]
    sub[inside] = colour


def photo_like(w: int, h: int, seed: int = 0, polygons: int = 200) -> np.ndarray:
    rng = SplitMix64(seed)
    base = rng.between(64, 192, 3)
    rgb = np.empty((h, w, 3), dtype=np.int64)
    for ch in range(3):
        rgb[:, :, ch] = base[ch]
    for cell, amp in ((64, 96), (32, 48), (16, 24), (8, 12)):
        shared = _value_noise(rng, w, h, cell, amp)
        for ch in range(3):
            own = _value_noise(rng, w, h, cell, amp)
            # a*S + b*X with a = 2, b = 1 gives correlation a^2/(a^2+b^2) = 0.8;
            # divide by sqrt(5) ~ 256/572 to keep the amplitude.
            rgb[:, :, ch] += ((2 * shared + own) * 229) >> 9
    for _ in range(polygons):
        cx = int(rng.below(w, 1)[0])
        cy = int(rng.below(h, 1)[0])
        r = int(rng.between(4, max(8, min(w, h) // 6), 1)[0])
        k = int(rng.between(3, 6, 1)[0])
        # convex polygon: vertices on a circle at sorted random angles (integer
        # sin/cos from a 64-entry table in 1.14 fixed point)
        ang = np.sort(rng.below(64, k))
        px = cx + ((r * _COS64[ang]) >> 14)
        py = cy + ((r * _SIN64[ang]) >> 14)
        colour = rng.between(0, 255, 3)
        _fill_polygon(rgb, np.stack([px, py], axis=1), colour)
    rgb += rng.between(-1, 1, w * h * 3).reshape(h, w, 3)
    return _to_bgra(rgb, np.full((h, w), 255, dtype=np.int64))


# 64-step circle in 1.14 fixed point: round(16384 * cos/sin(2 pi k / 64)).
_COS64 = np.array([
    16384, 16305, 16069, 15679, 15137, 14449, 13623, 12665, 11585, 10394, 9102, 7723, 6270, 4756, 3196, 1606,
    0, -1606, -3196, -4756, -6270, -7723, -9102, -10394, -11585, -12665, -13623, -14449, -15137, -15679, -16069, -16305,
    -16384, -16305, -16069, -15679, -15137, -14449, -13623, -12665, -11585, -10394, -9102, -7723, -6270, -4756, -3196, -1606,
    0, 1606, 3196, 4756, 6270, 7723, 9102, 10394, 11585, 12665, 13623, 14449, 15137, 15679, 16069, 16305,
], dtype=np.int64)
_SIN64 = np.roll(_COS64, 16)


def alpha_blobs(w: int, h: int, seed: int = 0) -> np.ndarray:
    rng = SplitMix64(seed)
    rgb = _gradient_noise_rgb(rng, w, h)
    # blob field: coarse value noise; the lowest ~30 % become alpha = 0, the
    # next ~15 % a smooth ramp, the rest opaque.
    field = _value_noise(rng, w, h, max(8, min(w, h) // 8), 1000) + _value_noise(rng, w, h, max(4, min(w, h) // 32), 250)
    flat = np.sort(field.reshape(-1))
    n = flat.size
    t0 = flat[min(n - 1, (n * 30) // 100)]
    t1 = flat[min(n - 1, (n * 45) // 100)]
    alpha = np.full((h, w), 255, dtype=np.int64)
    clear = field < t0
    ramp = (field >= t0) & (field < t1)
    span = max(int(t1 - t0), 1)
    alpha[ramp] = 1 + ((field[ramp] - t0) * 253) // span
    alpha[clear] = 0
    noise_rgb = rng.between(0, 255, w * h * 3).reshape(h, w, 3)
    rgb[clear] = noise_rgb[clear]
    return _to_bgra(rgb, alpha)


# round(65536 * 2 ** (j / 64)) for j in 0..63 (16.16 fixed point)
_EXP2_64 = np.array([
    65536, 66250, 66971, 67700, 68438, 69183, 69936, 70698, 71468, 72246, 73032, 73828, 74632, 75444, 76266, 77096,
    77936, 78785, 79642, 80510, 81386, 82273, 83169, 84074, 84990, 85915, 86851, 87796, 88752, 89719, 90696, 91684,
    92682, 93691, 94711, 95743, 96785, 97839, 98905, 99982, 101070, 102171, 103283, 104408, 105545, 106694, 107856, 109031,
    110218, 111418, 112631, 113858, 115098, 116351, 117618, 118899, 120194, 121502, 122825, 124163, 125515, 126882, 128263, 129660,
], dtype=np.int64)


def texture_sides(n: int, seed: int, lo: int, hi: int) -> np.ndarray:
    """n (w, h) pairs, each side log-uniform in [lo, hi] rounded up to x4.

    ``hi / lo`` must be a power of two; the exponent is drawn in 1/64-octave
    steps and evaluated with an integer table, so the result is exact.
    """
    octaves = (hi // lo).bit_length() - 1
    if lo << octaves != hi:
        raise ValueError("hi / lo must be a power of two")
    rng = SplitMix64(seed)
    e = rng.below(64 * octaves + 1, 2 * n)
    sides = (lo * _EXP2_64[e % 64] << (e // 64)) >> 16
    sides = np.clip(sides, lo, hi)
    sides = (sides + 3) & ~3
    return sides.reshape(n, 2)


def image_for(kind: str, w: int, h: int, seed: int) -> np.ndarray:
    if kind == "gradient_noise":
        return gradient_noise(w, h, seed)
    if kind == "photo_like":
        return photo_like(w, h, seed)
    if kind == "alpha_blobs":
        return alpha_blobs(w, h, seed)
    raise ValueError(f"unknown synthetic image kind {kind!r}")


def random_blocks(n: int, seed: int):
    """n independent 4x4 cells for block-level parity tests.

    Returns (cells, masks): uint8[n, 64] BGRA pixels (4 rows of 4) and
    uint8[n, 64] masks (bytes A,G,R,B per pixel).  Mixes noise, gradients,
    few-colour and edge blocks, near-solid and low-contrast blocks, opaque
    and translucent alpha, and masks with invisible pixels, all-invisible
    colour and arbitrary mask bytes.
    """
    rng = SplitMix64(seed)
    cells = np.zeros((n, 16, 4), dtype=np.int64)
    masks = np.full((n, 16, 4), 255, dtype=np.int64)
    kinds = rng.below(8, n)
    alpha_modes = rng.below(4, n)
    mask_modes = rng.below(7, n)
    for k in range(n):
        t = int(kinds[k])
        if t == 0:
            c = rng.below(256, 64).reshape(16, 4)
        elif t in (1, 5):
            a = rng.below(256, 4)
            b = rng.below(256, 4)
            wt = rng.below(65, 16) if t == 5 else (np.arange(16) * 64) // 15
            c = (a[None, :] * (64 - wt[:, None]) + b[None, :] * wt[:, None] + 32) >> 6
            amp = 8 if t == 5 else 2
            c = c + rng.between(-amp, amp, 64).reshape(16, 4)
        elif t in (2, 4, 6):
            npal = {2: int(rng.between(1, 3, 1)[0]), 4: 2, 6: 3}[t]
            pal = rng.below(256, 4 * npal).reshape(npal, 4)
            sel = rng.below(npal, 16)
            c = pal[sel]
            if t != 2:
                c = c + rng.between(-3, 3, 64).reshape(16, 4)
        elif t == 3:
            c = rng.below(256, 4)[None, :] + rng.between(-1, 1, 64).reshape(16, 4)
        else:
            c = rng.below(256, 4)[None, :] + rng.between(-6, 6, 64).reshape(16, 4)
        c = np.clip(c, 0, 255)
        am = int(alpha_modes[k])
        if am == 0:
            c[:, 3] = 255
        elif am == 1:
            c[:, 3] = 255 - rng.below(20, 16)
        cells[k] = c
        mm = int(mask_modes[k])
        if mm == 0:
            inv = rng.below(256, 16) < int(rng.below(256, 1)[0])
            masks[k, inv, 1:] = 0
        elif mm == 1:
            masks[k, :, 1:] = 0
        elif mm == 2:
            masks[k] = np.where(rng.below(5, 64).reshape(16, 4) == 0, 0, 255)
        elif mm == 3:
            masks[k] = rng.below(256, 64).reshape(16, 4)
    return cells.reshape(n, 64).astype(np.uint8), masks.reshape(n, 64).astype(np.uint8)


def random_start_blocks(n: int, seed: int) -> np.ndarray:
    """n arbitrary 16-byte starting blocks (any mode, any bits)."""
    rng = SplitMix64(seed)
    return rng.below(256, n * 16).reshape(n, 16).astype(np.uint8)


BATCH_PRESETS = ("draft", "default", "precise")


def batch_textures(n: int, seed: int, lo: int = 4, hi: int = 2048) -> list[dict]:
    """Descriptions of a mixed batch: n textures with sides log-uniform in
    [lo, hi] (rounded up to x4, non-square), 60 % opaque (photo-like or
    gradient + noise) and 40 % with alpha (blobs; encoded with the outline
    mask), presets draft / default / precise in equal shares.  Each entry:
    {"w", "h", "kind", "seed", "alpha", "preset"}.
    """
    sides = texture_sides(n, seed, lo, hi)
    rng = SplitMix64(seed ^ 0x5EED5EED)
    kind_draw = rng.below(100, n)
    preset_draw = rng.below(3, n)
    out = []
    for i in range(n):
        k = int(kind_draw[i])
        kind = "alpha_blobs" if k < 40 else ("photo_like" if k < 70 else "gradient_noise")
        out.append({"w": int(sides[i, 0]), "h": int(sides[i, 1]), "kind": kind, "seed": seed * 1000 + i,
                    "alpha": kind == "alpha_blobs", "preset": BATCH_PRESETS[int(preset_draw[i])]})
    return out
