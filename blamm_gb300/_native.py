"""ctypes bindings of the native libraries (no fallback: a missing library is an error)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_PKG, "_build")
GPU_LIB_PATH = os.path.join(BUILD_DIR, "libblamm_gpu.so")
HOST_LIB_PATH = os.path.join(BUILD_DIR, "libblamm_host.so")
CLI_PATH = os.path.join(_PKG, "bin", "blamm")

BLAMM_OK = 0
BLAMM_ERR_ARG = -1
BLAMM_ERR_CUDA = -2
BLAMM_ERR_OVERFLOW = -3
BLAMM_ERR_TIMEOUT = -4
BLAMM_ERR_NOMEM = -5
BLAMM_ERR_UNSUPPORTED = -6
BLAMM_ERR_STATE = -7

MODES = {"fp32": 0, "bf16": 1, "bf16x2": 2}

HIT_DTYPE = np.dtype([("pos", "<i8"), ("col", "<i4"), ("score", "<f4")])


class BlammError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"blamm error {code}: {msg}")
        self.code = code


class Stats(C.Structure):
    _fields_ = [("positions", C.c_int64), ("columns", C.c_int64), ("candidates", C.c_int64),
                ("hits", C.c_int64), ("tiles", C.c_int32), ("launches", C.c_int32),
                ("kernel_ms", C.c_float), ("total_ms", C.c_float)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


_gpu = None


def gpu_lib() -> C.CDLL:
    """Load libblamm_gpu.so (built by blamm_gb300.build); raises if it is missing."""
    global _gpu
    if _gpu is not None:
        return _gpu
    if not os.path.exists(GPU_LIB_PATH):
        raise ImportError(f"{GPU_LIB_PATH} is missing: run `python -m blamm_gb300.build` "
                          "(or __graft_entry__.build()) first")
    lib = C.CDLL(GPU_LIB_PATH)
    vp, i64, i32, f32p = C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_float)
    lib.blamm_version.restype = C.c_int
    lib.blamm_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
    lib.blamm_ctx_destroy.argtypes = [vp]
    lib.blamm_ctx_destroy.restype = None
    lib.blamm_last_error.argtypes = [vp]
    lib.blamm_last_error.restype = C.c_char_p
    lib.blamm_set_mode.argtypes = [vp, C.c_int]
    lib.blamm_set_motifs.argtypes = [vp, vp, C.c_int, C.c_int, vp, vp]
    lib.blamm_set_thresholds.argtypes = [vp, vp]
    lib.blamm_scan.argtypes = [vp, vp, i64, vp, i64, vp, i64, C.POINTER(i64)]
    lib.blamm_scan_device.argtypes = [vp, vp, i64, vp, i64, vp, i64, C.POINTER(i64)]
    lib.blamm_filter_score.argtypes = [vp, vp, C.c_int, C.c_int, vp, vp, vp, vp]
    lib.blamm_last_stats.argtypes = [vp, C.POINTER(Stats)]
    lib.blamm_debug_scores.argtypes = [vp, vp, i64, i64, i64, f32p]
    lib.blamm_guard_band.argtypes = [vp, f32p]
    for name in ("blamm_ctx_create", "blamm_set_mode", "blamm_set_motifs", "blamm_set_thresholds",
                 "blamm_scan", "blamm_scan_device", "blamm_filter_score", "blamm_last_stats",
                 "blamm_debug_scores", "blamm_guard_band"):
        getattr(lib, name).restype = C.c_int
    _ = i32
    _gpu = lib
    return lib


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class GpuScanner:
    """A device context with a resident motif bank (one per host thread)."""

    def __init__(self, device: int = 0, mode: str = "bf16x2"):
        self.lib = gpu_lib()
        h = C.c_void_p()
        rc = self.lib.blamm_ctx_create(device, C.byref(h))
        if rc != BLAMM_OK:
            raise BlammError(rc, f"cannot create a context on device {device}")
        self.h = h
        self.ncols = 0
        self.set_mode(mode)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.blamm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        if rc != BLAMM_OK:
            raise BlammError(rc, self.lib.blamm_last_error(self.h).decode())

    def set_mode(self, mode: str) -> None:
        self.mode = mode
        self._check(self.lib.blamm_set_mode(self.h, MODES[mode]))

    def set_motifs(self, P: np.ndarray, col_len: np.ndarray, thr: np.ndarray) -> None:
        """P: (ncols, p_rows) float32 -- column c of the reference's column-major P."""
        P = np.ascontiguousarray(P, dtype=np.float32)
        self._len = np.ascontiguousarray(col_len, dtype=np.int32)
        self._thr = np.ascontiguousarray(thr, dtype=np.float32)
        ncols, p_rows = P.shape
        self._check(self.lib.blamm_set_motifs(self.h, _ptr(P), p_rows, ncols, _ptr(self._len),
                                              _ptr(self._thr)))
        self.ncols = ncols

    def set_thresholds(self, thr: np.ndarray) -> None:
        self._thr = np.ascontiguousarray(thr, dtype=np.float32)
        self._check(self.lib.blamm_set_thresholds(self.h, _ptr(self._thr)))

    def scan(self, bases, run_start: np.ndarray, hit_cap: int | None = None) -> np.ndarray:
        """Scan a host stream; returns the hits (HIT_DTYPE), unordered."""
        b = np.frombuffer(bases, dtype=np.uint8) if isinstance(bases, (bytes, bytearray)) else bases
        b = np.ascontiguousarray(b, dtype=np.uint8)
        runs = np.ascontiguousarray(run_start, dtype=np.int64)
        cap = hit_cap if hit_cap is not None else max(1 << 16, len(b) * max(self.ncols, 1) // 2000)
        while True:
            out = np.empty(cap, dtype=HIT_DTYPE)
            nh = C.c_int64(0)
            rc = self.lib.blamm_scan(self.h, _ptr(b), len(b), _ptr(runs), len(runs), _ptr(out), cap,
                                     C.byref(nh))
            if rc == BLAMM_ERR_OVERFLOW and hit_cap is None:
                cap = int(nh.value * 1.1) + 1024
                continue
            self._check(rc)
            return out[: nh.value]

    def scan_device(self, d_bases: int, n: int, d_runs: int, nruns: int, d_hits: int,
                    hit_cap: int) -> int:
        """Device pointers in, device hits out; returns the hit count."""
        nh = C.c_int64(0)
        rc = self.lib.blamm_scan_device(self.h, C.c_void_p(d_bases), n, C.c_void_p(d_runs), nruns,
                                        C.c_void_p(d_hits), hit_cap, C.byref(nh))
        if rc == BLAMM_ERR_OVERFLOW:
            raise BlammError(rc, f"{nh.value} hits exceed the capacity {hit_cap}")
        self._check(rc)
        return nh.value

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.blamm_last_stats(self.h, C.byref(s)))
        return s.as_dict()

    def guard_band(self) -> np.ndarray:
        out = np.zeros(self.ncols, dtype=np.float32)
        self._check(self.lib.blamm_guard_band(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def debug_scores(self, bases, p0: int, npos: int) -> np.ndarray:
        b = np.ascontiguousarray(np.frombuffer(bases, dtype=np.uint8)
                                 if isinstance(bases, (bytes, bytearray)) else bases, dtype=np.uint8)
        out = np.zeros((npos, self.ncols), dtype=np.float32)
        self._check(self.lib.blamm_debug_scores(self.h, _ptr(b), len(b), p0, npos,
                                                out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def filter_score(self, d_R: int, m: int, n: int, d_thr: int, d_idx: int, d_score: int,
                     d_nocc: int) -> None:
        self._check(self.lib.blamm_filter_score(self.h, C.c_void_p(d_R), m, n, C.c_void_p(d_thr),
                                                C.c_void_p(d_idx), C.c_void_p(d_score),
                                                C.c_void_p(d_nocc)))
