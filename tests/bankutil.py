"""Shared helpers of the tests: random motif banks and streams, checked by the oracle."""
from __future__ import annotations

import numpy as np

import oracle
from blamm_gb300 import workloads


def make_bank(seed: int, nmotifs: int, lmin: int, lmax: int, rc: bool = True, rel: float = 0.8,
              bg=(300, 200, 200, 300), pseudo: float = 0.25, total: int = 100):
    """Motif bank as the reference builds it: motifs sorted by length, [fwd, rc] columns,
    PWMs from PFM2PWM, relative thresholds rel*(max-min)+min."""
    rng = np.random.default_rng(seed)
    pfms = workloads.random_pfms(rng, nmotifs, lmin, lmax, total=total)
    pfms.sort(key=lambda m: m[1].shape[0])
    cols = []
    for _, pfm in pfms:
        cols.append(oracle.pfm2pwm(pfm, bg, pseudo, False))
        if rc:
            cols.append(oracle.pfm2pwm(oracle.revcompl_pfm(pfm), bg, pseudo, True))
    lmaxc = max(c.shape[0] for c in cols)
    P = np.zeros((len(cols), 4 * lmaxc), dtype=np.float32)
    lens = np.zeros(len(cols), dtype=np.int32)
    thr = np.zeros(len(cols), dtype=np.float32)
    for i, pwm in enumerate(cols):
        P[i, :pwm.size] = pwm.reshape(-1)
        lens[i] = pwm.shape[0]
        mn, mx = oracle.min_max_score(pwm)
        thr[i] = np.float32(np.float32(rel) * np.float32(mx - mn) + np.float32(mn))
    return P, lens, thr


def make_stream(seed: int, n: int, nruns: int = 1, lower_frac: float = 0.0,
                probs=(0.3, 0.2, 0.2, 0.3)):
    """Random filtered stream with run starts and optional lowercase stretches."""
    rng = np.random.default_rng(seed)
    b = workloads.iid_bases(rng, n, probs)
    if lower_frac > 0 and n > 0:
        nseg = max(1, int(lower_frac * n / 50))
        for _ in range(nseg):
            s = int(rng.integers(0, n))
            b[s:s + int(rng.integers(1, 100))] |= 0x20
    if nruns > 1 and n > 1:
        starts = np.unique(rng.integers(1, n, size=nruns - 1))
        runs = np.concatenate([[0], starts]).astype(np.int64)
    else:
        runs = np.zeros(1, dtype=np.int64)
    return b, runs


def e4m3_round(x: np.ndarray) -> np.ndarray:
    """Nearest E4M3 value (3 mantissa bits, ties to even; subnormals on the grid 2^-9;
    |x| <= 448 assumed)."""
    a = np.abs(x)
    e = np.floor(np.log2(np.where(a > 0, a, 1.0)))
    ulp = np.where(a < 2.0 ** -6, 2.0 ** -9, 2.0 ** (e - 3))
    return np.sign(x) * np.round(a / ulp) * ulp


def quantized_columns(P: np.ndarray, lens: np.ndarray, terms: int) -> np.ndarray:
    """The terms the tensor cores see, as float64: fixed-point BF16 hi [+ lo] (terms 1, 2),
    or (terms 8) P x 2^k rounded to E4M3 with max |P| 2^k in (32, 64], divided by 2^k."""
    out = np.zeros(P.shape, dtype=np.float64)
    for c in range(P.shape[0]):
        v = P[c, :4 * lens[c]].astype(np.float64)
        mx = np.abs(v).max()
        if mx > 0:
            f, e = np.frexp(mx)
            e = int(e) - (1 if f == 0.5 else 0)
            e = max(-30, min(40, e))
        else:
            e = -30
        if terms == 8:
            k = 6 - e
            out[c, :4 * lens[c]] = e4m3_round(np.ldexp(v, k)) * 2.0 ** -k
            continue
        k = 7 - e
        hi = np.rint(np.ldexp(v, k)) * 2.0 ** -k
        q = hi
        if terms == 2:
            lo = np.rint(np.ldexp(v - hi, k + 8)) * 2.0 ** -(k + 8)
            q = hi + lo
        out[c, :4 * lens[c]] = q
    return out


def exact_window_scores(bases: np.ndarray, Q: np.ndarray, lens: np.ndarray, p0: int, npos: int):
    """sum_j Q[c, 4j + base(p+j)] for p in [p0, p0+npos), all columns, float64 (no run checks)."""
    n = len(bases)
    code = np.full(n + 512, 4, dtype=np.int64)
    up = {ord("A"): 0, ord("C"): 1, ord("G"): 2, ord("T"): 3}
    for ch, v in up.items():
        code[:n][bases == ch] = v
    ncols = Q.shape[0]
    out = np.zeros((npos, ncols), dtype=np.float64)
    Qz = np.concatenate([Q, np.zeros((ncols, 4))], axis=1)  # column 'code 4' -> 0 via index trick
    zero_idx = Q.shape[1]
    for c in range(ncols):
        L = int(lens[c])
        for j in range(L):
            b = code[p0 + j:p0 + j + npos]
            idx = np.where(b < 4, 4 * j + b, zero_idx)
            out[:, c] += Qz[c, idx]
    return out


def same_hits(a: np.ndarray, b: np.ndarray) -> tuple[bool, str]:
    a = np.sort(a, order=["pos", "col"])
    b = np.sort(b, order=["pos", "col"])
    if len(a) != len(b):
        sa = set(zip(a["pos"].tolist(), a["col"].tolist()))
        sb = set(zip(b["pos"].tolist(), b["col"].tolist()))
        return False, f"{len(a)} vs {len(b)} hits; only-first {sorted(sa - sb)[:5]} only-second {sorted(sb - sa)[:5]}"
    if not (np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["col"], b["col"])):
        return False, "different (pos, col) sets"
    if not np.array_equal(a["score"].view(np.uint32), b["score"].view(np.uint32)):
        i = int(np.flatnonzero(a["score"].view(np.uint32) != b["score"].view(np.uint32))[0])
        return False, f"score bits differ at {a[i]} vs {b[i]}"
    return True, f"{len(a)} identical hits"
