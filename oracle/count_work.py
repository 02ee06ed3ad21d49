#!/usr/bin/env python3
"""Counts the reference's algorithmic integer work per bench workload (test
infrastructure; writes oracle/work_counts.json, which bench.py reads for its
work roofline).

The counter build of the port (oracle/port_counters.h,
liboracle_port_counters.so) encodes each workload's whole image, step for
step as the reference does, and counts the terms its searches evaluate:

  subset errors      (pixel, level, channel) terms, 7 int ops each:
                     difference, absolute value, quantising shift, square,
                     weight multiply-add, level minimum, pixel sum;
  candidate scans    (window cell, pixel) table terms, 3 int ops each:
                     table read, square, sum;
  lower-bound scans  (cell, pixel) and (row, pixel) terms, 3 int ops each.

int_ops = 7 * err_terms + 3 * (scan_terms + est_terms).  These are the
operations of the reference's algorithm on this input; a GPU that
evaluates more candidates (lanes run ahead of an early exit) or spends
instructions on bookkeeping executes more.

Usage:  python oracle/count_work.py [workload ...]
"""

from __future__ import annotations

import ctypes
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT))

NAMES = ["err_calls", "err_terms", "scan_calls", "scan_terms", "est_calls", "est_terms"]
OPS = {"err_terms": 7, "scan_terms": 3, "est_terms": 3}


def main():
    import bench
    from oracle.pyoracle import HERE as OH, VP, I
    lib_path = OH / "liboracle_port_counters.so"
    if not lib_path.exists():
        import subprocess
        subprocess.run(["sh", str(OH / "build_oracle.sh")], check=True, stdout=subprocess.DEVNULL)
    L = ctypes.CDLL(str(lib_path))
    L.nebc7_oracle_compress_texture.argtypes = [VP, VP, VP, I, I, I, I, I, I, I, I, I, I, VP, VP]
    L.nebc7_oracle_init.argtypes = [I]
    L.nebc7_oracle_work.argtypes = [VP, I]
    names = sys.argv[1:] or list(bench.WORKLOADS)
    out_file = HERE / "work_counts.json"
    result = json.loads(out_file.read_text()) if out_file.exists() else {"workloads": {}}
    result["definition"] = "int_ops = 7 * err_terms + 3 * (scan_terms + est_terms); see oracle/count_work.py"
    threads = os.cpu_count() or 1
    for name in names:
        padded, mask, o, d, s, gkey = bench.prepare(name)
        ph, pw = padded.shape[:2]
        m = mask if mask is not None else np.full_like(padded, 255)
        out = np.zeros(((ph // 4) * (pw // 4), 16), np.uint8)
        err = np.zeros(2, np.int64)
        ssim = np.zeros(2, np.float64)
        L.nebc7_oracle_init(d)
        buf = np.zeros(len(NAMES), np.uint64)
        L.nebc7_oracle_work(buf.ctypes.data, 1)
        t = time.time()
        rc = L.nebc7_oracle_compress_texture(out.ctypes.data, padded.ctypes.data, m.ctypes.data, pw * 4, pw, ph, d, s,
                                             int(o["draft"]), int(o["normal"]), int(o["slow"]), int(o["linear"]),
                                             threads, err.ctypes.data, ssim.ctypes.data)
        assert rc == 0
        assert L.nebc7_oracle_work(buf.ctypes.data, 1) == len(NAMES)
        c = {k: int(v) for k, v in zip(NAMES, buf)}
        ops = sum(OPS[k] * c[k] for k in OPS)
        import hashlib
        golden = json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())["images"].get(gkey)
        exact = golden is not None and hashlib.sha256(out.tobytes()).hexdigest() == golden["output_sha256"]
        result["workloads"][name] = dict(c, int_ops=ops, blocks=int(out.shape[0]), int_ops_per_block=ops / out.shape[0],
                                         output_matches_golden=bool(exact))
        print(name, json.dumps(result["workloads"][name]), f"{time.time() - t:.1f}s", flush=True)
    out_file.write_text(json.dumps(result, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
