"""KTX 1.1 container of the reference's driver (CPU; the library is loaded
but no CUDA call is made)."""

import struct

import numpy as np
import pytest

from nebc7_gb300 import read_ktx, write_ktx, ktx_header


def _expected(w, h, flip):
    # KTX 1.1: identifier, endianness, glType 0, glTypeSize 1, glFormat 0,
    # GL_COMPRESSED_RGBA_BPTC_UNORM, GL_RGBA, w, h, depth 0, 0 array
    # elements, 1 face, 1 level, 28 bytes of key/value: one 23-byte pair
    # "KTXOrientation\0S=r,T=?\0" (the key spelled as the reference writes
    # it) + 1 pad byte, then the level's size
    ident = bytes([0xAB, 0x4B, 0x54, 0x58, 0x20, 0x31, 0x31, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A])
    pw, ph = (max(4, w) + 3) & ~3, (max(4, h) + 3) & ~3
    kv = b"KTXOrientation\x00S=r,T=" + (b"u" if flip else b"d") + b"\x00"
    return (ident + struct.pack("<13I", 0x04030201, 0, 1, 0, 0x8E8C, 0x1908, w, h, 0, 0, 1, 1, 28)
            + struct.pack("<I", len(kv)) + kv + b"\x00" + struct.pack("<I", pw * ph))


@pytest.mark.parametrize("w,h,flip", [(1024, 1024, False), (130, 98, True), (3, 5, False)])
def test_header_is_the_reference_layout(native, w, h, flip):
    assert ktx_header(w, h, flip) == _expected(w, h, flip)


def test_round_trip(native, tmp_path):
    blocks = np.arange(33 * 25 * 16, dtype=np.uint32).astype(np.uint8).reshape(-1, 16)   # 132 x 100 padded
    p = tmp_path / "t.ktx"
    write_ktx(str(p), blocks, 130, 98, flip=True)
    b2, w, h, flip = read_ktx(str(p))
    assert (w, h, flip) == (130, 98, True)
    assert np.array_equal(b2, blocks)
    with pytest.raises(ValueError):
        write_ktx(str(p), blocks[:-1], 130, 98)
