"""ctypes view of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
reference legs, always as the checker or the timed CPU baseline, never as part
of the product path.  Build with `make -C oracle` (or __graft_entry__.build()).
"""
from __future__ import annotations

import ctypes as C
import glob
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
CLI_PATH = os.path.join(HERE, "_build", "blamm_oracle")
REF_CLI_PATH = os.path.join(HERE, "_ref", "blamm")

HIT_DTYPE = np.dtype([("pos", "<i8"), ("col", "<i4"), ("score", "<f4")])

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} missing: run `make -C oracle`")
        L = C.CDLL(LIB_PATH)
        vp, i64 = C.c_void_p, C.c_int64
        L.orc_scan.argtypes = [vp, i64, vp, i64, vp, C.c_int, C.c_int, vp, vp, C.c_int, vp, i64]
        L.orc_scan.restype = i64
        L.orc_scan_ex.argtypes = [vp, i64, vp, i64, vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_int, vp, i64]
        L.orc_scan_ex.restype = i64
        L.orc_scan_blas.argtypes = [vp, i64, vp, i64, vp, C.c_int, C.c_int, vp, vp, vp, C.c_int,
                                    C.c_int, C.c_int, C.c_int, vp, i64]
        L.orc_scan_blas.restype = i64
        L.orc_set_blas.argtypes = [C.c_char_p]
        L.orc_set_blas.restype = C.c_int
        L.orc_pfm2pwm.argtypes = [vp, C.c_int, vp, C.c_float, C.c_int, vp]
        L.orc_pfm2pwm.restype = None
        L.orc_revcompl_pfm.argtypes = [vp, C.c_int, vp]
        L.orc_revcompl_pfm.restype = None
        L.orc_max_score.argtypes = [vp, C.c_int]
        L.orc_max_score.restype = C.c_float
        L.orc_min_score.argtypes = [vp, C.c_int]
        L.orc_min_score.restype = C.c_float
        L.orc_score_cutoff.argtypes = [vp, i64, C.c_float, C.c_float, C.c_float, C.c_float]
        L.orc_score_cutoff.restype = C.c_float
        L.orc_theoretical_hist.argtypes = [vp, C.c_int, vp, i64, C.c_uint64, vp]
        L.orc_theoretical_hist.restype = C.c_int
        L.orc_nucl_prob.argtypes = [vp, C.c_float, vp]
        L.orc_nucl_prob.restype = None
        L.orc_matrix_tiles.argtypes = [vp, C.c_int, i64, vp, C.c_int]
        L.orc_matrix_tiles.restype = C.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def pfm2pwm(pfm: np.ndarray, bg_counts, pseudo: float, revcomp: bool) -> np.ndarray:
    pfm = np.ascontiguousarray(pfm, dtype=np.uint64)
    bg = np.ascontiguousarray(bg_counts, dtype=np.uint64)
    out = np.zeros((pfm.shape[0], 4), dtype=np.float32)
    lib().orc_pfm2pwm(_p(pfm), pfm.shape[0], _p(bg), pseudo, int(revcomp), _p(out))
    return out


def revcompl_pfm(pfm: np.ndarray) -> np.ndarray:
    pfm = np.ascontiguousarray(pfm, dtype=np.uint64)
    out = np.zeros_like(pfm)
    lib().orc_revcompl_pfm(_p(pfm), pfm.shape[0], _p(out))
    return out


def min_max_score(pwm: np.ndarray) -> tuple[float, float]:
    pwm = np.ascontiguousarray(pwm, dtype=np.float32)
    return float(lib().orc_min_score(_p(pwm), pwm.shape[0])), float(lib().orc_max_score(_p(pwm), pwm.shape[0]))


def score_cutoff(counts, min_score: float, width: float, max_score: float, pvalue: float) -> float:
    c = np.ascontiguousarray(counts, dtype=np.uint64)
    return float(lib().orc_score_cutoff(_p(c), len(c), min_score, width, max_score, pvalue))


def theoretical_hist(pwm: np.ndarray, bg_prob, nbins: int, max_length: int) -> np.ndarray:
    pwm = np.ascontiguousarray(pwm, dtype=np.float32)
    bg = np.ascontiguousarray(bg_prob, dtype=np.float32)
    out = np.zeros(nbins, dtype=np.uint64)
    if lib().orc_theoretical_hist(_p(pwm), pwm.shape[0], _p(bg), nbins, max_length, _p(out)):
        raise RuntimeError("theoretical hist failed")
    return out


def nucl_prob(counts, pseudo: float) -> np.ndarray:
    c = np.ascontiguousarray(counts, dtype=np.uint64)
    out = np.zeros(4, dtype=np.float32)
    lib().orc_nucl_prob(_p(c), pseudo, _p(out))
    return out


def matrix_tiles(lens, min_zero_area: int) -> np.ndarray:
    lens = np.ascontiguousarray(lens, dtype=np.int32)
    out = np.zeros((2 * len(lens) + 4, 3), dtype=np.int32)
    n = lib().orc_matrix_tiles(_p(lens), len(lens), min_zero_area, _p(out), out.shape[0])
    return out[:n]


def motif_bank(pfms, bg_counts, pseudo: float = 0.25, pvalues=(1e-4,), nbins: int = 250,
               max_length: int = 10_000_000, revcompl: bool = True):
    """The reference's scan set-up for a list of PFMs, restated with the oracle's functions:
    motifs ordered by length (the sort in MotifContainer::loadCBMotifs / loadJasparMotifs,
    motif.cpp:367, 436), each followed by its reverse complement (addReverseComplements,
    motif.cpp:439-449), PWMs from the dictionary's base counts (PFM2PWM, motif.cpp:194-223),
    the matrix P (generateMatrix, motif.cpp:542-564) and per p-value thresholds from the
    theoretical histogram of each forward motif (hist.cpp:162-175, getScoreCutoff
    motif.cpp:47-69; a reverse complement shares its forward motif's histogram file,
    pwmscan.cpp:599-616).

    Returns (P (ncols x 4*Lmax), lengths, thresholds (len(pvalues) x ncols), column_motif,
    column_strand): column c scores PFM column_motif[c] on strand column_strand[c] (0 = +)."""
    order = sorted(range(len(pfms)), key=lambda i: np.asarray(pfms[i]).shape[0])
    bgp = nucl_prob(bg_counts, pseudo)
    cols = []
    for i in order:
        pfm = np.asarray(pfms[i])
        fwd = pfm2pwm(pfm, bg_counts, pseudo, False)
        mn, mx = min_max_score(fwd)
        width = np.float32(np.float32(mx) - np.float32(mn)) / np.float32(nbins)
        h = theoretical_hist(fwd, bgp, nbins, max_length)
        t = [score_cutoff(h, mn, float(width), mx, pv) for pv in pvalues]
        cols.append((fwd, i, 0, t))
        if revcompl:
            cols.append((pfm2pwm(revcompl_pfm(pfm), bg_counts, pseudo, True), i, 1, t))
    lmax = max(c[0].shape[0] for c in cols)
    P = np.zeros((len(cols), 4 * lmax), dtype=np.float32)
    for c, (pwm, _, _, _) in enumerate(cols):
        P[c, :pwm.size] = pwm.ravel()
    lens = np.array([c[0].shape[0] for c in cols], dtype=np.int32)
    thr = np.array([c[3] for c in cols], dtype=np.float32).T.copy()
    return (P, lens, thr, np.array([c[1] for c in cols], dtype=np.int64),
            np.array([c[2] for c in cols], dtype=np.int8))


def scan(bases: np.ndarray, run_start: np.ndarray, P: np.ndarray, col_len, thr,
         nthreads: int = 8, lower_scores: bool = False) -> np.ndarray:
    """Sequential-FP32 scan (the reference's hit set). P: (ncols, p_rows).
    lower_scores: lowercase bases score like uppercase (the simple scan, `scan -s`)."""
    b = np.ascontiguousarray(bases, dtype=np.uint8)
    runs = np.ascontiguousarray(run_start, dtype=np.int64)
    P = np.ascontiguousarray(P, dtype=np.float32)
    ln = np.ascontiguousarray(col_len, dtype=np.int32)
    th = np.ascontiguousarray(thr, dtype=np.float32)
    ncols, rows = P.shape
    args = (_p(b), len(b), _p(runs), len(runs), _p(P), rows, ncols, _p(ln), _p(th), nthreads, int(lower_scores))
    n = lib().orc_scan_ex(*args, None, 0)
    if n < 0:
        raise RuntimeError("oracle scan failed")
    out = np.zeros(n, dtype=HIT_DTYPE)
    lib().orc_scan_ex(*args, _p(out), n)
    return out


def find_blas() -> str | None:
    """scipy's LP64 OpenBLAS (the library the reference is linked against here)."""
    try:
        import scipy
    except ImportError:
        return None
    libs = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cands = [p for p in glob.glob(os.path.join(libs, "libscipy_openblas*.so*")) if "64_" not in p]
    return cands[0] if cands else None


_blas_ok = None


def scan_blas(bases: np.ndarray, run_start: np.ndarray, P: np.ndarray, col_len, thr, tiles,
              h: int = 1000, w: int = 250, nthreads: int = 8) -> np.ndarray:
    """The reference's own loop (one-hot S, per-offset sgemm per tile, threshold scan)."""
    global _blas_ok
    if _blas_ok is None:
        path = find_blas()
        _blas_ok = bool(path) and lib().orc_set_blas(path.encode()) == 0
    if not _blas_ok:
        raise RuntimeError("no LP64 BLAS available for the oracle's BLAS port")
    b = np.ascontiguousarray(bases, dtype=np.uint8)
    runs = np.ascontiguousarray(run_start, dtype=np.int64)
    P = np.ascontiguousarray(P, dtype=np.float32)
    ln = np.ascontiguousarray(col_len, dtype=np.int32)
    th = np.ascontiguousarray(thr, dtype=np.float32)
    tl = np.ascontiguousarray(tiles, dtype=np.int32)
    ncols, rows = P.shape
    args = (_p(b), len(b), _p(runs), len(runs), _p(P), rows, ncols, _p(ln), _p(th), _p(tl), len(tl),
            h, w, nthreads)
    n = lib().orc_scan_blas(*args, None, 0)
    if n < 0:
        raise RuntimeError("oracle BLAS scan failed")
    out = np.zeros(n, dtype=HIT_DTYPE)
    lib().orc_scan_blas(*args, _p(out), n)
    return out


def sort_hits(h: np.ndarray) -> np.ndarray:
    return np.sort(h, order=["pos", "col"])


def format_scores(values: np.ndarray) -> list[bytes]:
    """printf("%g") of each float (the reference's occurrence-file score text)."""
    v = np.ascontiguousarray(values, dtype=np.float32)
    out = C.create_string_buffer(32 * len(v))
    f = lib().orc_format_scores
    f.argtypes = [C.c_void_p, C.c_int64, C.c_char_p, C.c_int]
    f.restype = None
    f(_p(v), len(v), out, 32)
    raw = out.raw
    return [raw[32 * i:32 * i + 32].split(b"\0", 1)[0] for i in range(len(v))]
