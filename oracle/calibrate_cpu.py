#!/usr/bin/env python3
"""Calibrates the oracle port against the reference's own SIMD build on the
same CPU (test infrastructure: run on an x86-64 host where oracle/_ref/ is
built; writes oracle/cpu_calibration.json, which bench.py reads).

The GPU host is an Arm machine where the reference's SSE/AVX code cannot
build, so bench.py times the scalar port there.  This script times both CPU
encoders here on identical inputs -- the same blocks of the bench's
workloads, the same flags and preset, the same thread count, every core of
this host -- and records their throughputs and the ratio, so that the bench
line can state what the reference's SIMD path would do on the GPU host's
cores (the port's Arm figure times this ratio; an estimate, labelled so).

Each workload is sampled as evenly spaced block rows of its image (the
sample is named in the output); both encoders get the same cells and
masks through their block entries, best of three runs each.

Usage:  python oracle/calibrate_cpu.py [--threads N]
"""

from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT))

# workload -> (image kind, w, h, seed, flags, denoise, step, block-row spacing)
WORKLOADS = {
    "photo1024_draft": ("photo_like", 1024, 1024, 0, "/nomask /noflip /draft", 1, 9, 2),
    "photo1024_default": ("photo_like", 1024, 1024, 0, "/nomask /noflip", 1, 9, 4),
    "photo1024_precise": ("photo_like", 1024, 1024, 0, "/nomask /noflip", 0, 0, 8),
    "gradient256_default": ("gradient_noise", 256, 256, 0, "/nomask /noflip", 1, 9, 1),
    "alpha2048_slow": ("alpha_blobs", 2048, 2048, 0, "/noflip /slow", 1, 9, 16),
}


def cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def sample_cells(name):
    """Cells and masks (64 bytes each) of every spacing-th block row."""
    from nebc7_gb300 import synth
    from nebc7_gb300.api import outline_mask, pad_texture, parse_flags
    kind, w, h, seed, flags, d, s, spacing = WORKLOADS[name]
    o = parse_flags(flags)
    padded = pad_texture(synth.image_for(kind, w, h, seed))
    mask = outline_mask(padded, o["radius"]) if o["mask"] else np.full_like(padded, 255)
    ph, pw = padded.shape[:2]
    rows = list(range(0, ph // 4, spacing))
    def cells_of(a):
        band = a.reshape(ph // 4, 4, pw // 4, 4, 4)[rows]          # [row][y][bx][x][c]
        return np.ascontiguousarray(band.transpose(0, 2, 1, 3, 4).reshape(-1, 64))
    return cells_of(padded), cells_of(mask), o, d, s, f"{len(rows)} of {ph // 4} block rows (every {spacing}), " \
        f"{len(rows) * (pw // 4)} blocks of the {pw}x{ph} image"


def best_of(fn, runs=3):
    best = None
    for _ in range(runs):
        t = time.perf_counter()
        out = fn()
        dt = time.perf_counter() - t
        best = dt if best is None or dt < best else best
    return best, out


def main():
    from oracle.pyoracle import Port, Reference
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=str(HERE / "cpu_calibration.json"))
    args = ap.parse_args()
    port = Port()
    result = {"host": {"cpu": cpu_model(), "machine": platform.machine(), "threads": args.threads,
                       "reference_isa": "AVX2 + FMA + BMI2 (oracle/build_ref.sh)",
                       "port_build": "oracle/build_oracle.sh"},
              "workloads": {}}
    for name in WORKLOADS:
        cells, masks, o, d, s, sample = sample_cells(name)
        ref = Reference(d, s)
        n = len(cells)
        flags = (int(o["draft"]), int(o["normal"]), int(o["slow"]), int(o["linear"]))
        zero = np.zeros((n, 16), np.uint8)
        t_ref, (io_ref, e_ref) = best_of(lambda: (lambda io: (io, ref.compress_blocks(cells, masks, io, *flags,
                                                                                        threads=args.threads)))(zero.copy()))
        port.lib.nebc7_oracle_init(d)
        t_port, (io_port, e_port) = best_of(lambda: (lambda io: (io, port.compress_blocks(cells, masks, io, d, s, *flags,
                                                                                          threads=args.threads)))(zero.copy()))
        same = bool(np.array_equal(io_ref, io_port)) and e_ref[0].tolist() == e_port[0].tolist()
        px = n * 16
        entry = {"sample": sample, "blocks": n, "reference_mpx_s": px / t_ref / 1e6, "port_mpx_s": px / t_port / 1e6,
                 "port_time_over_reference": t_port / t_ref, "outputs_identical": same}
        result["workloads"][name] = entry
        print(name, json.dumps(entry), flush=True)
    Path(args.out).write_text(json.dumps(result, indent=1) + "\n")
    print("wrote", args.out)


if __name__ == "__main__":
    main()
