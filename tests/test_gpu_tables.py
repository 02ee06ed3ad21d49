"""The level tables the device builds (GPU) against the oracle port's, byte
for byte.

The port's tables are pinned to the reference build (tests/test_oracle_*,
tests/test_diff_tables.py).  Eleven device tables keep the reference's
per-x layout and must equal the port's copies exactly.  Three (the byte
table of 2-bit indices and the two nibble tables) are stored once, indexed
by endpoint differences; every x, cL, cH of the reference's per-x table must
read the same value from them.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = ["d2v8", "d2v7", "d2v6", "d2v5", "c2v8", "c2v6", "c2v5", "d3v7s", "d3v6", "d3v5", "c3v7s", "c3v5", "d4h", "d2h"]
BY_DIFFERENCES = {"d2v8": (256, False), "d4h": (256, True), "d2h": (256, True)}


def _device_table(native, denoise, which):
    n = ctypes.c_longlong()
    buf = np.zeros(1 << 23, np.uint8)
    assert native.nebc7_table_read(denoise, which, buf.ctypes.data, buf.nbytes, ctypes.byref(n)) == 0
    return buf[:n.value].copy()


def _port_table(port, denoise, which):
    n = ctypes.c_int()
    ptr = port.lib.nebc7_oracle_table(denoise, which, ctypes.byref(n))
    return np.frombuffer(ctypes.string_at(ptr, n.value), np.uint8)


@pytest.mark.parametrize("denoise", [0, 1])
@pytest.mark.parametrize("name", NAMES)
def test_device_table_equals_port(native, port, denoise, name):
    which = NAMES.index(name)
    dev = _device_table(native, denoise, which)
    ref = _port_table(port, denoise, which)
    if name not in BY_DIFFERENCES:
        assert dev.shape == ref.shape
        bad = np.nonzero(dev != ref)[0]
        assert len(bad) == 0, f"{name}: {len(bad)} bytes differ, first {bad[:8].tolist()}"
        return
    n, nibbles = BY_DIFFERENCES[name]
    c = np.arange(n)
    cH, cL = np.meshgrid(c, c, indexing="ij")
    if nibbles:
        diff = dev.reshape(511, 256)
        ref = np.stack([ref & 0xF, ref >> 4], axis=-1).reshape(256, n * n)
    else:
        diff = dev.reshape(511, 512)
        ref = ref.reshape(256, n * n)
    for x in range(256):
        a, b = cH - x + 255, cL - x + 255
        if nibbles:
            got = (diff[a, b >> 1] >> ((b & 1) * 4)) & 0xF
        else:
            got = diff[a, b]
        assert np.array_equal(got.reshape(-1), ref[x]), f"{name} x={x}"


def _expanded(bits):
    q = np.arange(1 << bits)
    return (q << (8 - bits)) | (q >> (2 * bits - 8)) if bits < 8 else q


@pytest.mark.parametrize("denoise", [0, 1])
@pytest.mark.parametrize("name,diff_index,bits", [("d2v7", 0, 7), ("d2v6", 0, 6), ("d2v5", 0, 5), ("d3v6", 14, 6),
                                                   ("d3v5", 14, 5)])
def test_reduced_tables_read_by_differences(native, port, denoise, name, diff_index, bits):
    """The encoder reads each reduced table of 2- or 3-bit indices as the
    device's difference table of that index width at the bit-replicated
    endpoints (d2v8, and d3v8 for 3-bit indices): every x, cL, cH gives the
    port's entry."""
    diff = _device_table(native, denoise, diff_index).reshape(511, 512)
    ref = _port_table(port, denoise, NAMES.index(name)).reshape(256, -1)
    e = _expanded(bits)
    eH, eL = np.meshgrid(e, e, indexing="ij")
    for x in range(256):
        got = diff[eH - x + 255, eL - x + 255].reshape(-1)
        assert np.array_equal(got, ref[x]), f"{name} x={x}"


def test_table_read_rejects_bad_arguments(native):
    n = ctypes.c_longlong()
    small = np.zeros(16, np.uint8)
    assert native.nebc7_table_read(1, 15, small.ctypes.data, small.nbytes, ctypes.byref(n)) == 1
    assert native.nebc7_table_read(2, 0, small.ctypes.data, small.nbytes, ctypes.byref(n)) == 1
    assert native.nebc7_table_read(1, 0, small.ctypes.data, small.nbytes, ctypes.byref(n)) == 6
    assert n.value == 511 * 512
