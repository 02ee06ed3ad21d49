"""Test infrastructure: ctypes bindings to the CPU oracles.

* ``Port``: the scalar restatement in this directory (liboracle_port.so),
  built on any host by oracle/build_oracle.sh; the checker of the parity
  tests and the CPU baseline of bench.py.
* ``Reference``: the reference encoder compiled from its own sources by
  oracle/build_ref.sh (x86 only, oracle/_ref/); used to pin ``Port`` and to
  generate the committed golden fixtures.
* ``ReferenceCli``: the reference's command-line build (its own
  configuration, the real job pool, the /map and /bad outputs).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this.
"""

from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "liboracle_port.so"
REF_DIR = HERE / "_ref"

VP, I = ctypes.c_void_p, ctypes.c_int


def _p(a):
    return None if a is None else a.ctypes.data


def build_port() -> Path:
    srcs = list(HERE.glob("port_*.cpp")) + list(HERE.glob("port_*.h"))
    if not PORT_LIB.exists() or any(s.stat().st_mtime > PORT_LIB.stat().st_mtime for s in srcs):
        subprocess.run(["sh", str(HERE / "build_oracle.sh")], check=True, stdout=subprocess.DEVNULL)
    return PORT_LIB


class Port:
    def __init__(self):
        build_port()
        L = ctypes.CDLL(str(PORT_LIB))
        L.nebc7_oracle_compress_blocks.argtypes = [VP, VP, VP, I, I, I, I, I, I, I, I, VP, VP]
        L.nebc7_oracle_compress_texture.argtypes = [VP, VP, VP, I, I, I, I, I, I, I, I, I, I, VP, VP]
        L.nebc7_oracle_decompress_blocks.argtypes = [VP, VP, I]
        L.nebc7_oracle_prepare_texture.argtypes = [VP, I, I, VP, VP, I]
        L.nebc7_oracle_init.argtypes = [I]
        L.nebc7_oracle_set_pca.argtypes = [I]
        L.nebc7_oracle_table.restype = VP
        L.nebc7_oracle_table.argtypes = [I, I, ctypes.POINTER(ctypes.c_int)]
        self.lib = L

    def compress_blocks(self, cells, masks, io, denoise, step, draft=1, normal=0, slow=0, linear=0, threads=1):
        err = np.zeros(2, np.int64)
        ssim = np.zeros(2, np.float64)
        rc = self.lib.nebc7_oracle_compress_blocks(_p(cells), _p(masks), _p(io), len(io), denoise, step,
                                                   draft, normal, slow, linear, threads, _p(err), _p(ssim))
        assert rc == 0
        return err, ssim

    def compress_texture(self, dst, padded, mask, denoise, step, draft=1, normal=0, slow=0, linear=0, threads=1):
        ph, pw = padded.shape[:2]
        err = np.zeros(2, np.int64)
        ssim = np.zeros(2, np.float64)
        rc = self.lib.nebc7_oracle_compress_texture(_p(dst), _p(padded), _p(mask), pw * 4, pw, ph, denoise, step,
                                                    draft, normal, slow, linear, threads, _p(err), _p(ssim))
        assert rc == 0
        return err, ssim

    def prepare(self, img, radius):
        h, w = img.shape[:2]
        pw, ph = (max(4, w) + 3) & ~3, (max(4, h) + 3) & ~3
        padded = np.zeros((ph, pw, 4), np.uint8)
        mask = np.zeros((ph, pw, 4), np.uint8)
        img = np.ascontiguousarray(img)
        assert self.lib.nebc7_oracle_prepare_texture(_p(img), w, h, _p(padded), _p(mask), radius) == 0
        return padded, mask

    def decompress_blocks(self, blocks):
        blocks = np.ascontiguousarray(blocks)
        out = np.zeros((len(blocks), 64), np.uint8)
        self.lib.nebc7_oracle_decompress_blocks(_p(blocks), _p(out), len(blocks))
        return out


class Reference:
    """The reference encoder built from its sources (one library per preset).
    variant "m6i2": its draft chain reduced to the Mode6Index2 pass
    (oracle/ref_m6i2_only.cpp; default preset only)."""

    def __init__(self, denoise: int, step: int, variant: str = ""):
        path = REF_DIR / f"libnebc7_ref_d{denoise}s{step}{'_' + variant if variant else ''}.so"
        if not path.exists():
            raise FileNotFoundError(f"{path} (run oracle/build_ref.sh on an x86-64 host with the reference sources)")
        L = ctypes.CDLL(str(path))
        L.nebc7_ref_compress_blocks.argtypes = [VP, VP, VP, I, I, I, I, I, I, VP, VP]
        L.nebc7_ref_decompress_blocks.argtypes = [VP, VP, I]
        L.nebc7_ref_encode_image.argtypes = [VP, I, I, ctypes.c_char_p, VP, VP, I, I, VP, VP]
        L.nebc7_ref_table.restype = VP
        L.nebc7_ref_table.argtypes = [I, ctypes.POINTER(ctypes.c_int)]
        self.lib = L

    def compress_blocks(self, cells, masks, io, draft=1, normal=0, slow=0, linear=0, threads=8):
        err = np.zeros(2, np.int64)
        ssim = np.zeros(2, np.float64)
        rc = self.lib.nebc7_ref_compress_blocks(_p(cells), _p(masks), _p(io), len(io), draft, normal, slow, linear,
                                                threads, _p(err), _p(ssim))
        assert rc == 0
        return err, ssim

    def encode_image(self, img, flags, threads=8, preload=None):
        h, w = img.shape[:2]
        pw, ph = (max(4, w) + 3) & ~3, (max(4, h) + 3) & ~3
        out = np.zeros(pw * ph, np.uint8) if preload is None else preload.copy()
        err = np.zeros(2, np.int64)
        ssim = np.zeros(2, np.float64)
        img = np.ascontiguousarray(img)
        rc = self.lib.nebc7_ref_encode_image(_p(img), w, h, flags.encode(), _p(preload), _p(out), out.size, threads,
                                             _p(err), _p(ssim))
        assert rc == 0, rc
        return out.reshape(-1, 16), err, ssim


class ReferenceCli:
    """The reference's command-line build (oracle/ref_cli_shim.h): runs its
    CLI driver on an in-memory image and returns the encoded blocks and the
    /map and /bad images (padded BGRA, top-down)."""

    def __init__(self):
        path = REF_DIR / "libnebc7_ref_cli.so"
        if not path.exists():
            raise FileNotFoundError(f"{path} (run oracle/build_ref.sh on an x86-64 host with the reference sources)")
        L = ctypes.CDLL(str(path))
        L.nebc7_ref_cli.argtypes = [VP, I, I, ctypes.c_char_p, VP, I, VP, VP]
        self.lib = L

    def run(self, img, flags):
        h, w = img.shape[:2]
        pw, ph = (max(4, w) + 3) & ~3, (max(4, h) + 3) & ~3
        blocks = np.zeros(pw * ph, np.uint8)
        mp = np.zeros((ph, pw, 4), np.uint8)
        bad = np.zeros((ph, pw, 4), np.uint8)
        img = np.ascontiguousarray(img)
        rc = self.lib.nebc7_ref_cli(_p(img), w, h, flags.encode(), _p(blocks), blocks.size, _p(mp), _p(bad))
        assert rc == 7, rc
        return blocks.reshape(-1, 16), mp, bad
