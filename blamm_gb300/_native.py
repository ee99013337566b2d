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

MODES = {"fp32": 0, "bf16": 1, "bf16x2": 2, "auto": 3, "e4m3": 4}

HIT_DTYPE = np.dtype([("pos", "<i8"), ("col", "<i4"), ("score", "<f4")])


class BlammError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"blamm error {code}: {msg}")
        self.code = code


class Stats(C.Structure):
    _fields_ = [("positions", C.c_int64), ("columns", C.c_int64), ("candidates", C.c_int64),
                ("hits", C.c_int64), ("tiles", C.c_int32), ("launches", C.c_int32),
                ("kernel_ms", C.c_float), ("total_ms", C.c_float), ("scan_ms", C.c_float),
                ("rescore_ms", C.c_float)]

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
    lib.blamm_ctx_stream.argtypes = [vp, C.POINTER(vp)]
    lib.blamm_device_count.argtypes = [C.POINTER(C.c_int)]
    lib.blamm_set_softmask.argtypes = [vp, C.c_int]
    lib.blamm_score_histograms.argtypes = [vp, vp, i64, vp, i64, vp, vp, C.c_int, vp]
    lib.blamm_debug_profile.argtypes = [vp, C.c_int]
    lib.blamm_debug_profile_read.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_int)]
    lib.blamm_scan_device_static.argtypes = [vp, vp, i64, vp, i64, vp, i64, C.POINTER(i64)]
    lib.blamm_set_columns.argtypes = [vp, vp, C.c_int]
    lib.blamm_reserve.argtypes = [vp, i64, i64]
    lib.blamm_scan_enqueue.argtypes = [vp, vp, i64, vp, i64, vp, i64, vp]
    lib.blamm_scan_graph_create.argtypes = [vp, vp, i64, vp, i64, vp, i64, vp, C.POINTER(vp)]
    lib.blamm_scan_graph_launch.argtypes = [vp, vp]
    lib.blamm_scan_graph_destroy.argtypes = [vp]
    lib.blamm_scan_graph_destroy.restype = None
    lib.blamm_autotune.argtypes = [vp, vp, i64, vp, i64, C.POINTER(C.c_float)]
    lib.blamm_theoretical_hist.argtypes = [vp, vp, C.c_int, C.c_int, vp, vp, vp, C.c_int, C.c_uint64, C.c_int,
                                           vp, C.c_int, vp, vp]
    lib.blamm_device_memory.argtypes = [C.c_int, C.POINTER(i64), C.POINTER(i64)]
    lib.blamm_set_plan_options.argtypes = [vp, C.c_int, C.c_float]
    lib.blamm_debug_stall.argtypes = [vp, C.c_int, C.c_longlong]
    lib.blamm_fasta_parse_device.argtypes = [vp, vp, i64, vp, C.POINTER(i64), vp, vp, vp, C.POINTER(i64), vp,
                                             C.POINTER(i64), vp]
    lib.blamm_get_plan_options.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_float)]
    lib.blamm_get_terms.argtypes = [vp]
    lib.blamm_ctx_call_bytes.argtypes = [vp, C.POINTER(i64)]
    lib.blamm_release_buffers.argtypes = [vp]
    lib.blamm_stream_load_fasta.argtypes = [vp, vp, i64, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), vp]
    lib.blamm_stream_tables.argtypes = [vp, vp, vp, vp, vp]
    lib.blamm_scan_stream.argtypes = [vp, i64, i64, vp, i64, vp, i64, C.POINTER(i64)]
    for name in ("blamm_ctx_create", "blamm_set_mode", "blamm_set_motifs", "blamm_set_thresholds",
                 "blamm_scan", "blamm_scan_device", "blamm_filter_score", "blamm_last_stats",
                 "blamm_debug_scores", "blamm_guard_band", "blamm_ctx_stream", "blamm_device_count",
                 "blamm_set_softmask", "blamm_score_histograms", "blamm_debug_profile",
                 "blamm_debug_profile_read", "blamm_scan_device_static", "blamm_set_columns",
                 "blamm_reserve", "blamm_scan_enqueue", "blamm_scan_graph_create", "blamm_scan_graph_launch",
                 "blamm_autotune", "blamm_theoretical_hist", "blamm_device_memory", "blamm_set_plan_options",
                 "blamm_get_plan_options", "blamm_fasta_parse_device", "blamm_debug_stall", "blamm_get_terms",
                 "blamm_ctx_call_bytes", "blamm_release_buffers", "blamm_stream_load_fasta",
                 "blamm_stream_tables", "blamm_scan_stream"):
        getattr(lib, name).restype = C.c_int
    _ = i32
    _gpu = lib
    return lib


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class GpuScanner:
    """A device context with a resident motif bank (one per host thread)."""

    def __init__(self, device: int = 0, mode: str = "auto"):
        self.lib = gpu_lib()
        h = C.c_void_p()
        rc = self.lib.blamm_ctx_create(device, C.byref(h))
        if rc != BLAMM_OK:
            raise BlammError(rc, f"cannot create a context on device {device}")
        self.h = h
        self.ncols = 0
        self._stream = (0, 0, 0)
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
                    hit_cap: int, overflow_ok: bool = False) -> int:
        """Device pointers in, device hits out; returns the hit count (with overflow_ok, a
        count above hit_cap instead of an error: only hit_cap hits were stored)."""
        nh = C.c_int64(0)
        rc = self.lib.blamm_scan_device(self.h, C.c_void_p(d_bases), n, C.c_void_p(d_runs), nruns,
                                        C.c_void_p(d_hits), hit_cap, C.byref(nh))
        if rc == BLAMM_ERR_OVERFLOW:
            if overflow_ok:
                return nh.value
            raise BlammError(rc, f"{nh.value} hits exceed the capacity {hit_cap}")
        self._check(rc)
        return nh.value

    def scan_device_static(self, d_bases: int, n: int, d_runs: int, nruns: int, d_hits: int,
                           hit_cap: int) -> int:
        """scan_device through the allocation-free entry point (library-owned fixed scratch)."""
        nh = C.c_int64(0)
        rc = self.lib.blamm_scan_device_static(self.h, C.c_void_p(d_bases), n, C.c_void_p(d_runs), nruns,
                                               C.c_void_p(d_hits), hit_cap, C.byref(nh))
        if rc == BLAMM_ERR_OVERFLOW:
            raise BlammError(rc, self.lib.blamm_last_error(self.h).decode())
        self._check(rc)
        return nh.value

    def set_columns(self, cols) -> None:
        """Scan only these bank columns (None or empty: all)."""
        if cols is None or len(cols) == 0:
            self._check(self.lib.blamm_set_columns(self.h, None, 0))
            return
        c = np.ascontiguousarray(cols, dtype=np.int32)
        self._check(self.lib.blamm_set_columns(self.h, _ptr(c), len(c)))

    def reserve(self, max_positions: int, max_candidates: int) -> None:
        self._check(self.lib.blamm_reserve(self.h, max_positions, max_candidates))

    def enqueue(self, d_bases: int, n: int, d_runs: int, nruns: int, d_hits: int, hit_cap: int,
                d_counts: int) -> None:
        """Enqueue a scan without host synchronisation; counts land in d_counts (4 x uint64)."""
        self._check(self.lib.blamm_scan_enqueue(self.h, C.c_void_p(d_bases), n, C.c_void_p(d_runs), nruns,
                                                C.c_void_p(d_hits), hit_cap, C.c_void_p(d_counts)))

    def graph_create(self, d_bases: int, n: int, d_runs: int, nruns: int, d_hits: int, hit_cap: int,
                     d_counts: int) -> int:
        g = C.c_void_p()
        self._check(self.lib.blamm_scan_graph_create(self.h, C.c_void_p(d_bases), n, C.c_void_p(d_runs), nruns,
                                                     C.c_void_p(d_hits), hit_cap, C.c_void_p(d_counts),
                                                     C.byref(g)))
        return g.value

    def graph_launch(self, graph: int) -> None:
        self._check(self.lib.blamm_scan_graph_launch(self.h, C.c_void_p(graph)))

    def graph_destroy(self, graph: int) -> None:
        self.lib.blamm_scan_graph_destroy(C.c_void_p(graph))

    def theoretical_hist(self, P: np.ndarray, col_len: np.ndarray, bg_prob, pvalues=(), hist_of=None,
                         nbins: int = 250, max_length: int = 10_000_000, fp64_dp: bool = False,
                         counts: bool = False):
        """GPU theoretical histograms: (thresholds (len(pvalues) x ncols), counts (ncols x nbins) or None)."""
        Pc = np.ascontiguousarray(P, dtype=np.float32)
        ln = np.ascontiguousarray(col_len, dtype=np.int32)
        ncols, p_rows = Pc.shape
        hof = None if hist_of is None else np.ascontiguousarray(hist_of, dtype=np.int32)
        bg = np.ascontiguousarray(bg_prob, dtype=np.float32)
        pv = np.ascontiguousarray(pvalues, dtype=np.float32)
        thr = np.zeros((len(pv), ncols), dtype=np.float32)
        cnt = np.zeros((ncols, nbins), dtype=np.uint64) if counts else None
        self._check(self.lib.blamm_theoretical_hist(
            self.h, _ptr(Pc), p_rows, ncols, _ptr(ln), _ptr(hof) if hof is not None else None, _ptr(bg), nbins,
            max_length, int(fp64_dp), _ptr(pv) if len(pv) else None, len(pv), _ptr(thr) if len(pv) else None,
            _ptr(cnt) if cnt is not None else None))
        return thr, cnt

    def fasta_parse_device(self, d_raw: int, nraw: int, d_bases: int, d_run_start: int, d_run_seq: int,
                           d_run_seqpos: int, d_header_pos: int, nucl: np.ndarray | None = None) -> tuple[int, int, int]:
        """GPU FASTA ingest into caller device buffers: (bases, runs, sequences); the stream's
        A/C/G/T counts go to `nucl` (uint64[4]) when given."""
        nb, nr, ns = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.lib.blamm_fasta_parse_device(
            self.h, C.c_void_p(d_raw), nraw, C.c_void_p(d_bases), C.byref(nb), C.c_void_p(d_run_start),
            C.c_void_p(d_run_seq), C.c_void_p(d_run_seqpos), C.byref(nr), C.c_void_p(d_header_pos), C.byref(ns),
            _ptr(nucl) if nucl is not None else None))
        return nb.value, nr.value, ns.value

    def stream_load_fasta(self, raw: bytes) -> tuple[int, int, int, np.ndarray]:
        """FASTA text (host bytes) parsed on the device into the resident stream:
        (bases, runs, sequences, A/C/G/T counts)."""
        buf = np.frombuffer(raw, dtype=np.uint8) if len(raw) else np.zeros(1, dtype=np.uint8)
        nb, nr, ns = C.c_int64(), C.c_int64(), C.c_int64()
        nucl = np.zeros(4, dtype=np.uint64)
        self._check(self.lib.blamm_stream_load_fasta(self.h, _ptr(buf), len(raw), C.byref(nb), C.byref(nr),
                                                     C.byref(ns), _ptr(nucl)))
        self._stream = (nb.value, nr.value, ns.value)
        return nb.value, nr.value, ns.value, nucl

    def stream_tables(self) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
        """The resident stream's run table (start, sequence, position in it) and header offsets."""
        _, nr, ns = self._stream
        rs, rq, rp = (np.zeros(max(nr, 1), dtype=np.int64) for _ in range(3))
        hp = np.zeros(max(ns, 1), dtype=np.int64)
        self._check(self.lib.blamm_stream_tables(self.h, _ptr(rs), _ptr(rq), _ptr(rp), _ptr(hp)))
        return rs[:nr], rq[:nr], rp[:nr], hp[:ns]

    def scan_stream(self, begin: int, n: int, run_start: np.ndarray, hit_cap: int | None = None) -> np.ndarray:
        """Scan positions [begin, begin + n) of the resident stream (runs relative to begin)."""
        runs = np.ascontiguousarray(run_start, dtype=np.int64)
        cap = hit_cap if hit_cap is not None else max(1 << 16, n * max(self.ncols, 1) // 2000)
        while True:
            out = np.empty(max(cap, 1), dtype=HIT_DTYPE)
            nh = C.c_int64(0)
            rc = self.lib.blamm_scan_stream(self.h, begin, n, _ptr(runs), len(runs), _ptr(out), cap, C.byref(nh))
            if rc == BLAMM_ERR_OVERFLOW and hit_cap is None:
                cap = int(nh.value * 1.1) + 1024
                continue
            self._check(rc)
            return out[:nh.value].copy()

    def debug_stall(self, enable: bool, wait_limit_cycles: int = 0) -> None:
        """Failure-path test hook (see blamm_debug_stall)."""
        self._check(self.lib.blamm_debug_stall(self.h, int(enable), wait_limit_cycles))

    def set_plan_options(self, max_tile_columns: int, job_cost: float) -> None:
        self._check(self.lib.blamm_set_plan_options(self.h, max_tile_columns, job_cost))

    def plan_options(self) -> tuple[int, float]:
        n, c = C.c_int(), C.c_float()
        self._check(self.lib.blamm_get_plan_options(self.h, C.byref(n), C.byref(c)))
        return n.value, c.value

    def call_bytes(self) -> int:
        """Device bytes of the per-call buffers the context keeps."""
        b = C.c_int64(0)
        self._check(self.lib.blamm_ctx_call_bytes(self.h, C.byref(b)))
        return b.value

    def release_buffers(self) -> None:
        self._check(self.lib.blamm_release_buffers(self.h))
        self._stream = (0, 0, 0)

    def terms(self) -> int:
        """BF16 terms of the tensor-core scan in the current mode (0 in FP32 mode)."""
        return int(self.lib.blamm_get_terms(self.h))

    def autotune(self, d_bases: int, n: int, d_runs: int, nruns: int) -> float:
        ms = C.c_float(0.0)
        self._check(self.lib.blamm_autotune(self.h, C.c_void_p(d_bases), n, C.c_void_p(d_runs), nruns,
                                            C.byref(ms)))
        return ms.value

    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        p = C.c_void_p()
        self._check(self.lib.blamm_ctx_stream(self.h, C.byref(p)))
        return p.value or 0

    def set_softmask(self, lowercase_scores: bool) -> None:
        self._check(self.lib.blamm_set_softmask(self.h, int(bool(lowercase_scores))))

    def score_histograms(self, bases, run_start, min_score, width, nbins: int) -> np.ndarray:
        b = np.ascontiguousarray(bases, dtype=np.uint8)
        runs = np.ascontiguousarray(run_start, dtype=np.int64)
        mn = np.ascontiguousarray(min_score, dtype=np.float32)
        w = np.ascontiguousarray(width, dtype=np.float32)
        out = np.zeros((self.ncols, nbins), dtype=np.uint64)
        self._check(self.lib.blamm_score_histograms(self.h, _ptr(b), len(b), _ptr(runs), len(runs), _ptr(mn),
                                                    _ptr(w), nbins, _ptr(out)))
        return out

    def profile(self, enable: bool) -> None:
        self._check(self.lib.blamm_debug_profile(self.h, int(enable)))

    def profile_read(self) -> np.ndarray:
        """Per-CTA role timing of the last tensor-core scan, shape (ctas, 32)."""
        n = C.c_int(0)
        self._check(self.lib.blamm_debug_profile_read(self.h, None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 32), dtype=np.int64)
        self._check(self.lib.blamm_debug_profile_read(self.h, _ptr(out), n.value, C.byref(n)))
        return out[: n.value]

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


# ---------------------------------------------------------------- host library
_host = None


def host_lib() -> C.CDLL:
    """Load libblamm_host.so (motif banks, PWMs, histograms); raises if it is missing."""
    global _host
    if _host is not None:
        return _host
    if not os.path.exists(HOST_LIB_PATH):
        raise ImportError(f"{HOST_LIB_PATH} is missing: run `python -m blamm_gb300.build` first")
    gpu_lib()  # dependency, loaded from the same directory
    lib = C.CDLL(HOST_LIB_PATH)
    vp = C.c_void_p
    lib.blamm_host_last_error.restype = C.c_char_p
    lib.blamm_bank_load.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(vp)]
    lib.blamm_bank_from_pfms.argtypes = [vp, vp, C.c_int, C.c_int, C.POINTER(vp)]
    lib.blamm_bank_free.argtypes = [vp]
    lib.blamm_bank_free.restype = None
    lib.blamm_bank_columns.argtypes = [vp]
    lib.blamm_bank_max_len.argtypes = [vp]
    lib.blamm_bank_generate.argtypes = [vp, vp, C.c_float]
    lib.blamm_bank_matrix.argtypes = [vp, vp, vp, vp]
    lib.blamm_bank_min_max.argtypes = [vp, vp, vp]
    lib.blamm_bank_pvalue_thresholds.argtypes = [vp, vp, C.c_int, C.c_uint64, C.c_float, vp]
    lib.blamm_format_scores.argtypes = [vp, C.c_int64, C.c_char_p, C.c_int]
    lib.blamm_format_scores.restype = C.c_int
    lib.blamm_bank_hist_columns.argtypes = [vp, vp]
    lib.blamm_bank_hist_columns.restype = C.c_int
    lib.blamm_bank_name.argtypes = [vp, C.c_int]
    lib.blamm_bank_name.restype = C.c_char_p
    for name in ("blamm_bank_load", "blamm_bank_from_pfms", "blamm_bank_columns", "blamm_bank_max_len",
                 "blamm_bank_generate", "blamm_bank_matrix", "blamm_bank_min_max",
                 "blamm_bank_pvalue_thresholds"):
        getattr(lib, name).restype = C.c_int
    i64 = C.c_int64
    lib.blamm_server_create.argtypes = [C.POINTER(ServerConfig), vp, C.c_int, C.c_int, vp, vp, C.c_int,
                                        C.POINTER(vp)]
    lib.blamm_server_submit.argtypes = [vp, vp, i64, vp, i64, vp, C.c_int, C.c_int, C.POINTER(i64)]
    lib.blamm_server_wait.argtypes = [vp, i64, i64, C.POINTER(i64), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
    lib.blamm_server_take.argtypes = [vp, i64, vp, i64, C.POINTER(i64)]
    lib.blamm_server_stats_get.argtypes = [vp, C.POINTER(ServerStats)]
    lib.blamm_server_last_error.argtypes = [vp]
    lib.blamm_server_last_error.restype = C.c_char_p
    lib.blamm_server_destroy.argtypes = [vp]
    lib.blamm_server_destroy.restype = None
    for name in ("blamm_server_create", "blamm_server_submit", "blamm_server_wait", "blamm_server_take",
                 "blamm_server_stats_get"):
        getattr(lib, name).restype = C.c_int
    _host = lib
    return lib


def format_scores(values: np.ndarray) -> list[bytes]:
    """Scores as the occurrence file prints them (the host library's formatter)."""
    v = np.ascontiguousarray(values, dtype=np.float32)
    out = C.create_string_buffer(32 * len(v))
    if host_lib().blamm_format_scores(_ptr(v), len(v), out, 32) != 0:
        raise BlammError(-1, "blamm_format_scores failed")
    raw = out.raw
    return [raw[32 * i:32 * i + 32].split(b"\0", 1)[0] for i in range(len(v))]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("slots", C.c_int), ("mode", C.c_int), ("hbm_budget", C.c_int64)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("queued", C.c_int64), ("bases", C.c_int64), ("bp_columns", C.c_double),
                ("bytes_in_flight", C.c_int64), ("bytes_held", C.c_int64), ("peak_committed", C.c_int64),
                ("budget", C.c_int64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class Server:
    """The scan service of include/blamm_serve.h: resident bank + threshold sets, `slots`
    requests in flight, admission by device memory."""

    def __init__(self, P: np.ndarray, col_len: np.ndarray, thr_sets: np.ndarray, slots: int = 4,
                 mode: str = "bf16x2", device: int = 0, hbm_budget: int = 0):
        self.lib = host_lib()
        Pc = np.ascontiguousarray(P, dtype=np.float32)  # (ncols, p_rows): column-major P
        ln = np.ascontiguousarray(col_len, dtype=np.int32)
        ts = np.ascontiguousarray(np.atleast_2d(thr_sets), dtype=np.float32)
        cfg = ServerConfig(device, slots, MODES[mode], hbm_budget)
        h = C.c_void_p()
        rc = self.lib.blamm_server_create(C.byref(cfg), _ptr(Pc), Pc.shape[1], Pc.shape[0], _ptr(ln), _ptr(ts),
                                          ts.shape[0], C.byref(h))
        if rc != BLAMM_OK:
            raise BlammError(rc, "cannot create the server")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.blamm_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        if rc != BLAMM_OK:
            raise BlammError(rc, self.lib.blamm_server_last_error(self.h).decode())

    def submit(self, bases, run_start, cols=None, thr_set: int = 0) -> int:
        b = np.ascontiguousarray(np.frombuffer(bases, dtype=np.uint8)
                                 if isinstance(bases, (bytes, bytearray)) else bases, dtype=np.uint8)
        r = np.ascontiguousarray(run_start, dtype=np.int64)
        c = None if cols is None or len(cols) == 0 else np.ascontiguousarray(cols, dtype=np.int32)
        rid = C.c_int64()
        self._check(self.lib.blamm_server_submit(self.h, _ptr(b), len(b), _ptr(r), len(r),
                                                 _ptr(c) if c is not None else None, 0 if c is None else len(c),
                                                 thr_set, C.byref(rid)))
        return rid.value

    def wait(self, rid: int, timeout_ms: int = -1) -> tuple[int, float, float]:
        """(hits, latency ms, queueing ms) of a finished request."""
        nh, lat, q = C.c_int64(), C.c_double(), C.c_double()
        self._check(self.lib.blamm_server_wait(self.h, rid, timeout_ms, C.byref(nh), C.byref(lat), C.byref(q)))
        return nh.value, lat.value, q.value

    def take(self, rid: int) -> np.ndarray:
        nh, _, _ = self.wait(rid)
        out = np.empty(max(nh, 1), dtype=HIT_DTYPE)
        n = C.c_int64()
        self._check(self.lib.blamm_server_take(self.h, rid, out.ctypes.data_as(C.c_void_p), len(out), C.byref(n)))
        return out[: n.value]

    def stats(self) -> dict:
        st = ServerStats()
        self._check(self.lib.blamm_server_stats_get(self.h, C.byref(st)))
        return st.as_dict()


class MotifBank:
    """A MotifContainer of the host library (sorted by length, optional rc columns)."""

    def __init__(self, handle: C.c_void_p):
        self.lib = host_lib()
        self.h = handle

    @classmethod
    def load(cls, motif_file: str, permutations: bool = True, revcompl: bool = True) -> "MotifBank":
        lib = host_lib()
        h = C.c_void_p()
        if lib.blamm_bank_load(motif_file.encode(), int(permutations), int(revcompl), C.byref(h)) != 0:
            raise BlammError(-1, lib.blamm_host_last_error().decode())
        return cls(h)

    @classmethod
    def from_pfms(cls, pfms: list[np.ndarray], revcompl: bool = True) -> "MotifBank":
        lib = host_lib()
        lens = np.array([p.shape[0] for p in pfms], dtype=np.int32)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(p, dtype=np.uint64).reshape(-1, 4) for p in pfms]))
        h = C.c_void_p()
        if lib.blamm_bank_from_pfms(_ptr(flat), _ptr(lens), len(pfms), int(revcompl), C.byref(h)) != 0:
            raise BlammError(-1, lib.blamm_host_last_error().decode())
        return cls(h)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.blamm_bank_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def columns(self) -> int:
        return self.lib.blamm_bank_columns(self.h)

    @property
    def max_len(self) -> int:
        return self.lib.blamm_bank_max_len(self.h)

    def generate(self, bg_counts, pseudo: float = 0.25) -> None:
        bg = np.ascontiguousarray(bg_counts, dtype=np.uint64)
        if self.lib.blamm_bank_generate(self.h, _ptr(bg), pseudo) != 0:
            raise BlammError(-1, self.lib.blamm_host_last_error().decode())

    def matrix(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(P as (columns, 4*max_len) float32, lengths, rc flags) after generate()."""
        n, L = self.columns, self.max_len
        P = np.zeros((n, 4 * L), dtype=np.float32)
        lens = np.zeros(n, dtype=np.int32)
        rc = np.zeros(n, dtype=np.int32)
        self.lib.blamm_bank_matrix(self.h, _ptr(P), _ptr(lens), _ptr(rc))
        return P, lens, rc

    def min_max(self) -> tuple[np.ndarray, np.ndarray]:
        mn = np.zeros(self.columns, dtype=np.float32)
        mx = np.zeros(self.columns, dtype=np.float32)
        self.lib.blamm_bank_min_max(self.h, _ptr(mn), _ptr(mx))
        return mn, mx

    def pvalue_thresholds(self, bg_prob, pvalue: float, nbins: int = 250,
                          max_length: int = 10_000_000) -> np.ndarray:
        bg = np.ascontiguousarray(bg_prob, dtype=np.float32)
        thr = np.zeros(self.columns, dtype=np.float32)
        if self.lib.blamm_bank_pvalue_thresholds(self.h, _ptr(bg), nbins, max_length, pvalue, _ptr(thr)) != 0:
            raise BlammError(-1, self.lib.blamm_host_last_error().decode())
        return thr

    def hist_columns(self) -> np.ndarray:
        """Per column, the forward column whose histogram gives its threshold."""
        out = np.zeros(self.columns, dtype=np.int32)
        if self.lib.blamm_bank_hist_columns(self.h, _ptr(out)) != 0:
            raise BlammError(-1, self.lib.blamm_host_last_error().decode())
        return out

    def name(self, c: int) -> str:
        return self.lib.blamm_bank_name(self.h, c).decode()


class FastaReader:
    """Chunks of the filtered base stream of FASTA files (host library)."""

    def __init__(self, files: list[str], max_filt: int = -1):
        self.lib = host_lib()
        L = self.lib
        vp, i64 = C.c_void_p, C.c_int64
        L.blamm_fasta_open.argtypes = [C.POINTER(C.c_char_p), C.c_int, i64, C.POINTER(vp)]
        L.blamm_fasta_open.restype = C.c_int
        L.blamm_fasta_next.argtypes = [vp, i64, i64, C.POINTER(vp), C.POINTER(i64), C.POINTER(i64),
                                       C.POINTER(i64), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp),
                                       C.POINTER(i64)]
        L.blamm_fasta_next.restype = C.c_int
        L.blamm_fasta_num_sequences.argtypes = [vp]
        L.blamm_fasta_num_sequences.restype = i64
        L.blamm_fasta_sequence_name.argtypes = [vp, i64]
        L.blamm_fasta_sequence_name.restype = C.c_char_p
        L.blamm_fasta_close.argtypes = [vp]
        L.blamm_fasta_close.restype = None
        arr = (C.c_char_p * len(files))(*[f.encode() for f in files])
        self.h = C.c_void_p()
        if L.blamm_fasta_open(arr, len(files), max_filt, C.byref(self.h)) != 0:
            raise BlammError(-1, L.blamm_host_last_error().decode())

    def next_chunk(self, payload: int, overlap: int):
        """(offset, payload, bases uint8, markers (k, 3) int64) or None at the end."""
        b, mp, ms, mq = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        size, pay, off, nm = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        rc = self.lib.blamm_fasta_next(self.h, payload, overlap, C.byref(b), C.byref(size), C.byref(pay),
                                       C.byref(off), C.byref(mp), C.byref(ms), C.byref(mq), C.byref(nm))
        if rc < 0:
            raise BlammError(rc, self.lib.blamm_host_last_error().decode())
        if rc == 0:
            return None
        bases = np.ctypeslib.as_array(C.cast(b, C.POINTER(C.c_uint8)), (size.value,)).copy() if size.value else \
            np.zeros(0, np.uint8)
        k = nm.value
        cols = [np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int64)), (k,)).copy() for p in (mp, ms, mq)]
        return off.value, pay.value, bases, np.stack(cols, axis=1)

    def sequence_names(self) -> list[str]:
        n = self.lib.blamm_fasta_num_sequences(self.h)
        return [self.lib.blamm_fasta_sequence_name(self.h, i).decode() for i in range(n)]

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.blamm_fasta_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
