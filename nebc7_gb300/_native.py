"""Build and load the CUDA library (in-tree, plain nvcc; no torch types).

The shared library ``nebc7_gb300/_lib/libnebc7_gb300.so`` exports the C ABI of
``include/nebc7_gb300.h``.  It is built for sm_103a only.  Loading fails loudly
when it is missing: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import threading
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libnebc7_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]

_lock = threading.Lock()
_lib = None


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build nebc7_gb300")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "nebc7_gb300.h"]


def needs_build() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    return any(p.stat().st_mtime > t for p in sources())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the CUDA library for sm_103a (a no-op when up to date)."""
    with _lock:
        if not force and not needs_build():
            return LIB
        objdir = LIBDIR / "obj"
        objdir.mkdir(parents=True, exist_ok=True)
        # one translation unit per encode instantiation: compiled in parallel
        procs = []
        objs = []
        for src in sorted(CSRC.glob("*.cu")):
            obj = objdir / (src.stem + ".o")
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((src, subprocess.Popen(cmd)))
            objs.append(obj)
        failed = [src.name for src, p in procs if p.wait() != 0]
        if failed:
            raise RuntimeError(f"nvcc failed on {', '.join(failed)}")
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", *map(str, objs), "-o", str(tmp)]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
        return LIB


# ---- ctypes bindings ----------------------------------------------------

VP = ctypes.c_void_p
I = ctypes.c_int
LL = ctypes.c_longlong


class Settings(ctypes.Structure):
    """nebc7_settings: the reference preset and InitTables flags."""

    _fields_ = [
        ("denoise", I),
        ("denoiseStep", I),
        ("doDraft", I),
        ("doNormal", I),
        ("doSlow", I),
        ("linearData", I),
    ]


class WorkerItem(ctypes.Structure):
    _fields_ = [("_Output", VP), ("_Cell", VP), ("_Mask", VP)]


class BlockSSIM(ctypes.Structure):
    _fields_ = [("Alpha", ctypes.c_double), ("Color", ctypes.c_double)]


class Texture(ctypes.Structure):
    """nebc7_texture: one texture of a batch (device buffers)."""

    _fields_ = [
        ("d_dst", VP),
        ("d_bgra", VP),
        ("d_mask", VP),
        ("stride", LL),
        ("w", I),
        ("h", I),
        ("settings", Settings),
    ]


BATCH_FROM_SCRATCH = 1


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_size_t), ("max_batch", I), ("streams", I)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("status", I), ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("errs", ctypes.c_int64 * 2), ("ssim", ctypes.c_double * 2), ("submit_at_ms", ctypes.c_double),
                ("launch_at_ms", ctypes.c_double), ("done_at_ms", ctypes.c_double), ("slot", I), ("launch", LL)]


class ServerCounters(ctypes.Structure):
    _fields_ = [("completed", LL), ("failed", LL), ("launches", LL), ("queued", LL), ("bytes_in_use", LL),
                ("peak_bytes", LL)]

PInitTables = ctypes.CFUNCTYPE(None, ctypes.c_bool, ctypes.c_bool, ctypes.c_bool, ctypes.c_bool)
PBlockKernel = ctypes.CFUNCTYPE(None, ctypes.POINTER(WorkerItem), ctypes.POINTER(WorkerItem), I,
                                ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(BlockSSIM))
PGetWeight = ctypes.CFUNCTYPE(I)


class IBc7Core(ctypes.Structure):
    _fields_ = [
        ("pInitTables", PInitTables),
        ("pDecompress", PBlockKernel),
        ("pCompress", PBlockKernel),
        ("pGetWeightAlpha", PGetWeight),
        ("pGetWeightColor", PGetWeight),
    ]


# name -> (restype, argtypes); every symbol declared in include/nebc7_gb300.h
SIGNATURES = {
    "nebc7_GetBc7Core": (ctypes.c_bool, [VP]),
    "nebc7_ProcessTexture": (None, [VP, VP, VP, I, I, I, VP, ctypes.c_size_t, VP, VP, VP]),
    "nebc7_set_preset": (I, [I, I]),
    "nebc7_last_error": (I, []),
    "nebc7_encode_device": (I, [VP, VP, VP, LL, I, I, ctypes.POINTER(Settings), VP, VP, VP]),
    "nebc7_encode_host": (I, [VP, VP, VP, LL, I, I, ctypes.POINTER(Settings), VP, VP]),
    "nebc7_encode_blocks_host": (I, [VP, VP, VP, I, ctypes.POINTER(Settings), VP, VP]),
    "nebc7_decode_device": (I, [VP, VP, LL, I, I, VP]),
    "nebc7_decode_blocks_host": (I, [VP, VP, I]),
    "nebc7_init_device": (I, [I]),
    "nebc7_encode_launches": (I, [ctypes.POINTER(Settings)]),
    "nebc7_set_pca": (I, [I]),
    "nebc7_table_read": (I, [I, I, VP, LL, ctypes.POINTER(LL)]),
    "nebc7_launch_shape": (I, [VP, VP, VP]),
    "nebc7_encode_device_noalloc": (I, [VP, VP, VP, LL, I, I, ctypes.POINTER(Settings), VP, VP]),
    "nebc7_batch_create": (I, [VP, I, I, VP]),
    "nebc7_batch_tune": (I, [VP, I, VP]),
    "nebc7_batch_launch": (I, [VP, VP]),
    "nebc7_batch_sums": (I, [VP, VP, VP, VP]),
    "nebc7_batch_set_schedule": (I, [VP, I]),
    "nebc7_batch_info": (I, [VP, VP, VP, VP]),
    "nebc7_batch_plan": (I, [VP, VP, VP, VP]),
    "nebc7_batch_set_plan": (I, [VP, I, I, I]),
    "nebc7_batch_trials": (I, [VP, VP, VP, VP, VP, I]),
    "nebc7_batch_destroy": (None, [VP]),
    "nebc7_server_create": (I, [VP, VP]),
    "nebc7_server_submit": (I, [VP, VP, VP, LL, I, I, ctypes.POINTER(Settings), VP, VP]),
    "nebc7_server_wait": (I, [VP, ctypes.c_int64, ctypes.c_double, VP]),
    "nebc7_server_stats": (I, [VP, VP]),
    "nebc7_server_destroy": (None, [VP]),
    "nebc7_prepare_device": (I, [VP, LL, I, I, VP, VP, I, VP]),
    "nebc7_bad_blocks_device": (I, [VP, VP, VP, LL, I, I, I, VP, VP]),
    "nebc7_partition_map_device": (I, [VP, VP, I, VP]),
    "nebc7_ktx_header": (I, [I, I, I, VP]),
}


def load(path: Path | None = None) -> ctypes.CDLL:
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else LIB
        if not p.exists():
            raise RuntimeError(
                f"nebc7_gb300 CUDA library not found at {p}; run nebc7_gb300.build() "
                "(there is no CPU fallback)")
        lib = ctypes.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


class NativeError(RuntimeError):
    CODES = {
        1: "invalid argument",
        2: "CUDA call failed",
        3: "device memory allocation failed",
        4: "pass not compiled into the library",
        5: "device iteration limit reached",
        6: "request exceeds a fixed capacity",
    }

    def __init__(self, code: int, what: str = ""):
        super().__init__(f"nebc7_gb300 error {code} ({self.CODES.get(code, 'unknown')}){': ' + what if what else ''}")
        self.code = code


def check(code: int, what: str = "") -> None:
    if code != 0:
        raise NativeError(code, what)
