"""The level tables with 8-bit endpoints, indexed by differences, hold the
reference's (x, c) entries (CPU).

The reference builds these tables per channel value x and endpoint pair
c = (cH << 8) + cL (src/Bc7Tables.cpp:643-776): the quantised distance from x
to the nearest interpolated level; the 4-bit ("half") tables clamp it to 15.
The device keeps one 511 x 511 table per kind, indexed by
(cH - x + 255, cL - x + 255), instead.  This checks, for every x, cL, cH, both
kDenoise values, the nibble tables of 2- and 4-bit indices and the byte table
of 2-bit indices, that the builders' formula over differences gives the
reference's entry.
"""

import numpy as np
import pytest

WEIGHTS = {4: (0, 21, 43, 64), 8: (0, 9, 18, 27, 37, 46, 55, 64),
           16: (0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64)}


def _quantise(d, denoise, clamp):
    q = d >> denoise if denoise else np.minimum(d, 127)
    return np.minimum(q, 15) if clamp else q


def _reference_rows(levels, denoise, clamp=True):
    """[x][cH][cL] as the reference defines it (per x)."""
    cL = np.arange(256, dtype=np.int32)[None, :]
    cH = np.arange(256, dtype=np.int32)[:, None]
    out = np.empty((256, 256, 256), np.uint8)
    interp = [((64 - w) * cL + w * cH + 32) >> 6 for w in WEIGHTS[levels]]
    for x in range(256):
        best = np.min(np.stack([np.abs(v - x) for v in interp]), axis=0)
        out[x] = _quantise(best, denoise, clamp)
    return out


def _difference_table(levels, denoise, clamp=True):
    """[a][b], a = cH - x + 255, b = cL - x + 255, as the device builder fills it."""
    a = np.arange(511, dtype=np.int32)[:, None]
    b = np.arange(511, dtype=np.int32)[None, :]
    dist = [np.abs((b - 255) + (((a - b) * w + 32) >> 6)) for w in WEIGHTS[levels]]
    return _quantise(np.min(np.stack(dist), axis=0), denoise, clamp).astype(np.uint8)


@pytest.mark.parametrize("levels,clamp", [(4, True), (16, True), (4, False)])
@pytest.mark.parametrize("denoise", [0, 1])
def test_difference_table_matches_reference_rows(levels, clamp, denoise):
    ref = _reference_rows(levels, denoise, clamp)
    diff = _difference_table(levels, denoise, clamp)
    cL = np.arange(256)[None, :]
    cH = np.arange(256)[:, None]
    for x in range(256):
        got = diff[cH - x + 255, cL - x + 255]
        assert np.array_equal(got, ref[x]), f"x={x}"


def test_difference_table_nibble_packing():
    # byte a * 256 + bb holds b = 2 bb in its low nibble and 2 bb + 1 in its high one
    diff = _difference_table(4, 1)
    padded = np.concatenate([diff, np.zeros((511, 1), np.uint8)], axis=1)
    packed = padded[:, 0::2] | (padded[:, 1::2] << 4)
    assert packed.shape == (511, 256)
    a, b = 300, 277
    assert (packed[a, b >> 1] >> ((b & 1) * 4)) & 0xF == diff[a, b]


def test_byte_table_row_layout():
    # rows of 512 bytes: byte (a << 9) + b, column 511 unused
    diff = _difference_table(4, 0, clamp=False)
    rows = np.zeros((511, 512), np.uint8)
    rows[:, :511] = diff
    flat = rows.reshape(-1)
    x, cL, cH = 17, 200, 3
    a, b = cH - x + 255, cL - x + 255
    assert flat[(a << 9) + b] == _reference_rows(4, 0, clamp=False)[x][cH, cL]


# (table id in the port, index levels, endpoint bits, shared p-bit, nibbles)
PORT_TABLES = {
    "d2v8": (0, 4, 8, False, False), "d2v7": (1, 4, 7, False, False), "d2v6": (2, 4, 6, False, False),
    "d2v5": (3, 4, 5, False, False), "d3v7s": (7, 8, 7, True, False), "d3v6": (8, 8, 6, False, False),
    "d3v5": (9, 8, 5, False, False), "d4h": (12, 16, 8, False, True), "d2h": (13, 4, 8, False, True),
}


def _port_table(denoise, tid):
    import ctypes
    from oracle.pyoracle import Port
    p = Port()
    n = ctypes.c_int()
    ptr = p.lib.nebc7_oracle_table(denoise, tid, ctypes.byref(n))
    return np.frombuffer(ctypes.string_at(ptr, n.value), np.uint8)


@pytest.mark.parametrize("denoise", [0, 1])
@pytest.mark.parametrize("name", sorted(PORT_TABLES))
def test_reference_tables_from_difference_tables(denoise, name):
    """Every byte and nibble table of the reference (as the port holds it,
    pinned to the reference build) is the difference table of its index
    width read at the bit-replicated endpoints, with a shared table's pairs
    of different parity marked 0xFF."""
    tid, levels, bits, shared, nibbles = PORT_TABLES[name]
    diff = _difference_table(levels, denoise, clamp=nibbles)
    n = 1 << bits
    ref = _port_table(denoise, tid)
    if nibbles:
        ref = np.stack([ref & 0xF, ref >> 4], axis=-1).reshape(256, n * n)
    else:
        ref = ref.reshape(256, n * n)
    q = np.arange(n)
    e = (q << (8 - bits)) + ((q << (8 - bits)) >> bits)
    qH, qL = np.meshgrid(q, q, indexing="ij")
    eH, eL = e[qH], e[qL]
    marked = shared & (((qH ^ qL) & 1) == 1)
    xs = range(256) if n <= 128 else range(0, 256, 5)
    for x in xs:
        got = np.where(marked, 0xFF, diff[eH - x + 255, eL - x + 255]).reshape(-1)
        assert np.array_equal(got, ref[x]), f"{name} x={x}"
