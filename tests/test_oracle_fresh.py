"""CPU tests: the oracle port against the reference built from its sources,
on inputs that are not in the committed fixtures.

The golden fixtures pin the port on fixed seeds.  Here both run side by side
on fresh seeds, for every preset the GPU path supports, from zero and from
random starting blocks, and on whole images through the driver steps
(padding, outline mask).  The reference libraries exist only on an x86-64
host with the reference sources (oracle/build_ref.sh); elsewhere these
tests skip.
"""

import numpy as np
import pytest

from nebc7_gb300 import synth

# (denoise, step, draft, normal, slow, linear, blocks)
PRESETS = {
    "d1s9_draft": (1, 9, 1, 0, 0, 0, 1024),
    "d1s9_normal": (1, 9, 1, 1, 0, 0, 256),
    "d1s9_slow": (1, 9, 1, 1, 1, 0, 128),
    "d1s9_linear": (1, 9, 1, 1, 0, 1, 48),
    "d0s0_normal": (0, 0, 1, 1, 0, 0, 160),
    "d0s0_slow": (0, 0, 1, 1, 1, 0, 96),
    "d1s0_normal": (1, 0, 1, 1, 0, 0, 256),
    "d0s9_normal": (0, 9, 1, 1, 0, 0, 256),
    "d1s9_m6i2": (1, 9, 2, 0, 0, 0, 1024),
}
SEEDS = [9001]


def _reference(denoise, step, draft=1):
    """The reference build of a preset; draft 2 (the Mode6Index2 fast run)
    is its m6i2 variant run with doDraft set."""
    from oracle.pyoracle import REF_DIR, Reference
    variant = "m6i2" if draft == 2 else ""
    if not (REF_DIR / f"libnebc7_ref_d{denoise}s{step}{'_' + variant if variant else ''}.so").exists():
        pytest.skip("reference build not present (x86 host with the reference sources only)")
    return Reference(denoise, step, variant)


@pytest.mark.parametrize("seed", SEEDS)
@pytest.mark.parametrize("start", ["zero", "random"])
@pytest.mark.parametrize("name", sorted(PRESETS))
def test_port_matches_reference_on_fresh_blocks(port, name, start, seed):
    d, s, draft, normal, slow, linear, n = PRESETS[name]
    ref = _reference(d, s, draft)
    cells, masks = synth.random_blocks(n, seed)
    starts = synth.random_start_blocks(n, seed + 1) if start == "random" else np.zeros((n, 16), np.uint8)
    io_ref = starts.copy()
    err_ref, ssim_ref = ref.compress_blocks(cells, masks, io_ref, min(draft, 1), normal, slow, linear, threads=8)
    io_port = starts.copy()
    err_port, ssim_port = port.compress_blocks(cells, masks, io_port, d, s, draft, normal, slow, linear, threads=8)
    differ = int(np.count_nonzero((io_port != io_ref).any(1)))
    assert differ == 0, f"{differ} of {n} blocks differ"
    assert err_port.tolist() == err_ref.tolist()
    assert np.allclose(ssim_port, ssim_ref, rtol=1e-12, atol=0)


IMAGES = [
    # kind, w, h, seed, flags, denoise, step
    ("alpha_blobs", 60, 44, 31, "/noflip", 1, 9),
    ("alpha_blobs", 32, 24, 32, "/noflip /slow", 1, 9),
    ("photo_like", 42, 21, 33, "/nomask /noflip", 0, 0),
    ("gradient_noise", 37, 29, 34, "/noflip /draft", 1, 9),
    ("gradient_noise", 16, 12, 35, "/nomask /noflip /data", 1, 9),
    ("alpha_blobs", 28, 20, 36, "/noflip /retina", 0, 0),
    ("alpha_blobs", 64, 40, 37, "/noflip /m6i2", 1, 9),
]


@pytest.mark.parametrize("case", IMAGES, ids=lambda c: f"{c[0]}_{c[1]}x{c[2]}_{c[4].replace('/', '').replace(' ', '_')}")
def test_port_matches_reference_on_fresh_images(port, case):
    from nebc7_gb300.api import parse_flags
    kind, w, h, seed, flags, d, s = case
    o = parse_flags(flags)
    ref = _reference(d, s, o["draft"])
    img = synth.image_for(kind, w, h, seed)
    out_ref, err_ref, ssim_ref = ref.encode_image(img, flags.replace("/m6i2", "/draft"))
    o = parse_flags(flags)
    padded, mask = port.prepare(img, o["radius"] if o["mask"] else -1)
    out = np.zeros((padded.shape[0] // 4 * (padded.shape[1] // 4), 16), np.uint8)
    err, ssim = port.compress_texture(out, padded, mask, d, s, int(o["draft"]), int(o["normal"]), int(o["slow"]),
                                      int(o["linear"]), threads=8)
    assert np.array_equal(out, out_ref)
    assert err.tolist() == err_ref.tolist()
    assert np.allclose(ssim, ssim_ref, rtol=1e-12, atol=0)
