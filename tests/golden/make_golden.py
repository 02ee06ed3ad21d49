"""Generates the golden fixtures from the reference encoder itself.

Runs the reference CPU encoder -- compiled from its own sources by
oracle/build_ref.sh into oracle/_ref/ (x86-64 only) -- on seeded synthetic
inputs and records its outputs:

* blocks_<set>.npz: outputs, error sums and SSIM sums for random 4x4 cells
  (nebc7_gb300.synth.random_blocks) under each preset / flag set, from zero
  starting blocks and from arbitrary starting blocks;
* golden.json: SHA-256 of the full BC7 payload plus error / SSIM sums for
  whole images run through the reference CLI driver (padding, masks, flags);
* tools_<name>.npz: the blocks and the /map and /bad images of the
  reference's command-line build (oracle/ref_cli_harness.cpp).

Usage:  python tests/golden/make_golden.py [name ...]   (needs oracle/_ref/*.so;
        with names, only those entries are made and the rest kept)
"""

from __future__ import annotations

import hashlib
import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from nebc7_gb300 import synth  # noqa: E402
from oracle.pyoracle import Reference  # noqa: E402

# name -> (denoise, step, draft, normal, slow, linear, start)
BLOCK_SETS = {
    "d1s9_draft": (1, 9, 1, 0, 0, 0, "zero"),
    "d1s9_normal": (1, 9, 1, 1, 0, 0, "zero"),
    "d1s9_slow": (1, 9, 1, 1, 1, 0, "zero"),
    "d1s9_linear": (1, 9, 1, 1, 0, 1, "zero"),
    "d1s9_normal_restart": (1, 9, 1, 1, 0, 0, "random"),
    "d1s9_draft_restart": (1, 9, 1, 0, 0, 0, "random"),
    "d0s0_draft": (0, 0, 1, 0, 0, 0, "zero"),
    "d0s0_normal": (0, 0, 1, 1, 0, 0, "zero"),
    "d0s0_slow": (0, 0, 1, 1, 1, 0, "zero"),
    "d1s0_normal": (1, 0, 1, 1, 0, 0, "zero"),
    "d0s9_normal": (0, 9, 1, 1, 0, 0, "zero"),
    # draft = 2: the "Mode6Index2 fast" run, from the reference's m6i2 variant
    # (oracle/ref_m6i2_only.cpp) with doDraft set and doNormal clear
    "d1s9_m6i2": (1, 9, 2, 0, 0, 0, "zero"),
    "d1s9_m6i2_restart": (1, 9, 2, 0, 0, 0, "random"),
}
BLOCKS_N = 512
BLOCKS_SEED = 20261203

# name -> (kind, w, h, seed, flags, denoise, step)
IMAGES = {
    "cfg1_256_default": ("gradient_noise", 256, 256, 0, "/nomask /noflip", 1, 9),
    "cfg1_256_draft": ("gradient_noise", 256, 256, 0, "/nomask /noflip /draft", 1, 9),
    "cfg2_1024_draft": ("photo_like", 1024, 1024, 0, "/nomask /noflip /draft", 1, 9),
    "cfg2_1024_default": ("photo_like", 1024, 1024, 0, "/nomask /noflip", 1, 9),
    "cfg2_1024_precise": ("photo_like", 1024, 1024, 0, "/nomask /noflip", 0, 0),
    "cfg3_2048_slow": ("alpha_blobs", 2048, 2048, 0, "/noflip /slow", 1, 9),
    "cfg3_2048_data": ("alpha_blobs", 2048, 2048, 0, "/data /noflip", 1, 9),
    "odd_130x98_default": ("photo_like", 130, 98, 2, "/nomask /noflip", 1, 9),
    "alpha_256_mask": ("alpha_blobs", 256, 256, 3, "/noflip", 1, 9),
    "alpha_256_retina_precise": ("alpha_blobs", 256, 256, 3, "/noflip /retina", 0, 0),
    "tiny_3x5_default": ("photo_like", 3, 5, 4, "/noflip", 1, 9),
    # /m6i2: the CLI's /draft on the reference's m6i2 variant
    "cfg2_1024_m6i2": ("photo_like", 1024, 1024, 0, "/nomask /noflip /m6i2", 1, 9),
    "alpha_256_m6i2": ("alpha_blobs", 256, 256, 3, "/noflip /m6i2", 1, 9),
}


# /map and /bad outputs of the reference CLI build (its own default preset):
# name -> (kind, w, h, seed, flags)
TOOLS = {
    "tools_alpha_96x64_draft": ("alpha_blobs", 96, 64, 8, "/noflip /draft"),
    "tools_alpha_96x64_data": ("alpha_blobs", 96, 64, 8, "/noflip /data /draft"),
    "tools_photo_64_default": ("photo_like", 64, 64, 9, "/nomask /noflip"),
    "tools_alpha_62x46_slow": ("alpha_blobs", 62, 46, 1, "/noflip /slow"),
}


def reference_for(d, s, draft):
    return Reference(d, s, "m6i2") if draft == 2 else Reference(d, s)


def reference_flags(flags):
    """The reference CLI has no /m6i2: it is /draft on the m6i2 variant."""
    return flags.replace("/m6i2", "/draft")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    cells, masks = synth.random_blocks(BLOCKS_N, BLOCKS_SEED)
    starts = synth.random_start_blocks(BLOCKS_N, BLOCKS_SEED + 1)
    meta = {
        "blocks": {"n": BLOCKS_N, "seed": BLOCKS_SEED, "cells_sha256": sha(cells), "masks_sha256": sha(masks),
                   "starts_sha256": sha(starts), "sets": {}},
        "images": {},
    }
    only = set(sys.argv[1:])
    if only:
        meta = json.loads((HERE / "golden.json").read_text())
    for name, (d, s, dr, no, sl, lin, start) in BLOCK_SETS.items():
        if only and name not in only:
            continue
        ref = reference_for(d, s, dr)
        io = np.zeros((BLOCKS_N, 16), np.uint8) if start == "zero" else starts.copy()
        t = time.time()
        err, ssim = ref.compress_blocks(cells, masks, io, min(dr, 1), no, sl, lin)
        np.savez_compressed(HERE / f"blocks_{name}.npz", out=io, err=err, ssim=ssim)
        meta["blocks"]["sets"][name] = {"denoise": d, "step": s, "draft": dr, "normal": no, "slow": sl,
                                        "linear": lin, "start": start, "err": err.tolist(), "ssim": ssim.tolist()}
        print(f"blocks {name}: {time.time() - t:.1f}s", flush=True)
    for name, (kind, w, h, seed, flags, d, s) in IMAGES.items():
        if only and name not in only:
            continue
        img = synth.image_for(kind, w, h, seed)
        ref = reference_for(d, s, 2 if "/m6i2" in flags else 1)
        t = time.time()
        out, err, ssim = ref.encode_image(img, reference_flags(flags))
        meta["images"][name] = {"kind": kind, "w": w, "h": h, "seed": seed, "flags": flags, "denoise": d, "step": s,
                                "input_sha256": sha(img), "output_sha256": sha(out), "err": err.tolist(),
                                "ssim": ssim.tolist(), "blocks": int(out.shape[0])}
        if out.shape[0] <= 4096:
            np.savez_compressed(HERE / f"image_{name}.npz", out=out)
        print(f"image {name}: {time.time() - t:.1f}s", flush=True)
    meta.setdefault("tools", {})
    for name, (kind, w, h, seed, flags) in TOOLS.items():
        if only and name not in only:
            continue
        from oracle.pyoracle import ReferenceCli
        img = synth.image_for(kind, w, h, seed)
        blocks, mp, bad = ReferenceCli().run(img, flags)
        np.savez_compressed(HERE / f"{name}.npz", blocks=blocks, map=mp, bad=bad)
        meta["tools"][name] = {"kind": kind, "w": w, "h": h, "seed": seed, "flags": flags, "denoise": 1, "step": 9,
                               "blocks_sha256": sha(blocks), "map_sha256": sha(mp), "bad_sha256": sha(bad),
                               "bad_blocks": int(bad.reshape(bad.shape[0] // 4, 4, bad.shape[1] // 4, 4, 4)
                                                 .any(axis=(1, 3, 4)).sum())}
        print(f"tools {name}", flush=True)
    (HERE / "golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
