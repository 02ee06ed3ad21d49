"""CPU tests: the /bad and /map restatements (oracle/pytools.py) and the
port against the reference's command-line build.

tests/golden/tools_*.npz hold what the reference's CLI driver writes with
/map and /bad on (tests/golden/make_golden.py, oracle/ref_cli_harness.cpp):
its blocks, the decoded partition visualisation and the glitch map.  These
pin the numpy restatements that the device kernels are tested against, and
the reference's own job pool and configuration against the port.
"""

import numpy as np
import pytest

from nebc7_gb300 import synth
from oracle import pytools

from conftest import GOLDEN

NAMES = ["tools_alpha_96x64_draft", "tools_alpha_96x64_data", "tools_photo_64_default", "tools_alpha_62x46_slow"]


def blocks_to_image(px, ph, pw):
    """Decoded blocks (n, 64 bytes: 4 rows of 4 BGRA pixels) -> uint8[ph, pw, 4]."""
    return np.ascontiguousarray(px.reshape(ph // 4, pw // 4, 4, 4, 4).transpose(0, 2, 1, 3, 4).reshape(ph, pw, 4))


def _case(port, golden, name):
    from nebc7_gb300.api import parse_flags
    g = golden["tools"][name]
    f = np.load(GOLDEN / f"{name}.npz")
    img = synth.image_for(g["kind"], g["w"], g["h"], g["seed"])
    o = parse_flags(g["flags"])
    padded, mask = port.prepare(img, o["radius"] if o["mask"] else -1)
    return g, f, o, padded, (mask if o["mask"] else None)


@pytest.mark.parametrize("name", NAMES)
def test_bad_map_restatement_matches_reference(port, golden, name):
    g, f, o, padded, mask = _case(port, golden, name)
    ph, pw = padded.shape[:2]
    dec = blocks_to_image(port.decompress_blocks(f["blocks"]), ph, pw)
    got = pytools.bad_blocks(padded, dec, mask, bool(o["linear"]))
    assert np.array_equal(got, f["bad"])
    assert int(got.reshape(ph // 4, 4, pw // 4, 4, 4).any(axis=(1, 3, 4)).sum()) == g["bad_blocks"] > 0


@pytest.mark.parametrize("name", NAMES)
def test_partition_map_restatement_matches_reference(port, golden, name):
    g, f, o, padded, mask = _case(port, golden, name)
    ph, pw = padded.shape[:2]
    vis = pytools.partition_map(f["blocks"])
    assert np.array_equal(blocks_to_image(port.decompress_blocks(vis), ph, pw), f["map"])


@pytest.mark.parametrize("name", NAMES)
def test_port_matches_reference_cli_blocks(port, golden, name):
    """The reference's CLI build (its own configuration and job pool) gives
    the blocks the port gives for the default preset."""
    g, f, o, padded, mask = _case(port, golden, name)
    ph, pw = padded.shape[:2]
    out = np.zeros(((ph // 4) * (pw // 4), 16), np.uint8)
    m = mask if mask is not None else np.full_like(padded, 255)
    port.compress_texture(out, padded, m, 1, 9, int(o["draft"]), int(o["normal"]), int(o["slow"]), int(o["linear"]),
                          threads=8)
    assert np.array_equal(out, f["blocks"])


def test_pca_bounds_prune_the_search():
    """OPTION_PCA's bounds only skip searches (src/Bc7CoreMode6.cpp:1407-1408:
    a full search runs when the bound is below the best error): with them on,
    the counter build of the port evaluates fewer subset-error terms on the
    same /slow blocks, and switching them off again restores the count."""
    import ctypes
    import subprocess
    from oracle.pyoracle import HERE as OH, VP, I
    lib_path = OH / "liboracle_port_counters.so"
    if not lib_path.exists():
        subprocess.run(["sh", str(OH / "build_oracle.sh")], check=True, stdout=subprocess.DEVNULL)
    L = ctypes.CDLL(str(lib_path))
    L.nebc7_oracle_init.argtypes = [I]
    L.nebc7_oracle_set_pca.argtypes = [I]
    L.nebc7_oracle_work.argtypes = [VP, I]
    L.nebc7_oracle_compress_blocks.argtypes = [VP, VP, VP, I, I, I, I, I, I, I, I, VP, VP]
    cells, masks = synth.random_blocks(300, 77)
    terms = []
    try:
        for on in (0, 1, 0):
            L.nebc7_oracle_set_pca(on)
            io = np.zeros((300, 16), np.uint8)
            err = np.zeros(2, np.int64)
            ssim = np.zeros(2, np.float64)
            w = np.zeros(6, np.uint64)
            L.nebc7_oracle_work(w.ctypes.data, 1)
            assert L.nebc7_oracle_compress_blocks(cells.ctypes.data, masks.ctypes.data, io.ctypes.data, 300, 1, 9,
                                                  1, 1, 1, 0, 8, err.ctypes.data, ssim.ctypes.data) == 0
            L.nebc7_oracle_work(w.ctypes.data, 0)
            terms.append(int(w[1]))
    finally:
        L.nebc7_oracle_set_pca(0)
    assert terms[1] < terms[0]
    assert terms[2] == terms[0]
