"""Lane check of tcgen05.mma kind::f8f6f4 (E4M3 operands, FP32 accumulate) on one CTA.

The one-term FP8 form of the scan would quantise P to E4M3 with a per-column scale: its
entries then span many binades (2^-9 .. 2^8 of the scale) and the guard band assumes that
the tensor cores add a k-step's products without losing bits.  This test runs one MMA
(M = 128, N = 32, K = 32) of tests/fp8_lane_check.cu on chosen operands:

* one-hot rows of A pick single entries of B: the operand layout;
* rows with four ones (one motif position per 4 K slots, the scan's one-hot pattern over
  8 positions) against B entries of mixed magnitudes: the sums the scan would form;
* rows of 32 ones against one large entry and many small ones: how far below the largest
  term the sum keeps bits.

All three are exact on GB300 (the one-term FP8 scan's guard band relies on it: a k-step adds
eight products, each an E4M3 value, into an FP32 accumulator that holds every partial sum
exactly).
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(os.path.dirname(HERE), "blamm_gb300", "_build")


def _e4m3_table() -> np.ndarray:
    """Value of each E4M3 code (sign, 4 exponent bits with bias 7, 3 mantissa bits;
    exponent 0 is subnormal, 0x7F and 0xFF are NaN)."""
    v = np.zeros(256)
    for code in range(256):
        s = -1.0 if code & 0x80 else 1.0
        e, m = (code >> 3) & 0xF, code & 7
        if e == 15 and m == 7:
            v[code] = np.nan
        elif e == 0:
            v[code] = s * m * 2.0 ** -9
        else:
            v[code] = s * (1 + m / 8) * 2.0 ** (e - 7)
    return v


E4M3 = _e4m3_table()
ONE = 0x38


def _lib():
    out = os.path.join(BUILD, "libfp8_lane_check.so")
    src = os.path.join(HERE, "fp8_lane_check.cu")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        os.makedirs(BUILD, exist_ok=True)
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared", "-Xcompiler", "-fPIC",
                        "-o", out, src], check=True)
    L = C.CDLL(out)
    L.fp8_lane_check.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.fp8_lane_check.restype = C.c_int
    return L


def _run(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.uint8)
    B = np.ascontiguousarray(B, dtype=np.uint8)
    assert A.shape == (128, 32) and B.shape == (32, 32)
    D = np.zeros((128, 32), dtype=np.float32)
    rc = _lib().fp8_lane_check(A.ctypes.data, B.ctypes.data, D.ctypes.data)
    assert rc == 0, f"lane check returned {rc}"
    return D


def _exact(A, B) -> np.ndarray:
    return E4M3[A] @ E4M3[B].T


def _finite_codes(rng, n, lo=0x01, hi=0x7E):
    c = rng.integers(lo, hi + 1, size=n).astype(np.uint8)
    return c | (rng.integers(0, 2, size=n).astype(np.uint8) << 7)


def test_one_hot_rows_select_single_entries():
    rng = np.random.default_rng(1)
    A = np.zeros((128, 32), dtype=np.uint8)
    A[np.arange(128), np.arange(128) % 32] = ONE
    B = _finite_codes(rng, 32 * 32).reshape(32, 32)
    D = _run(A, B)
    assert np.array_equal(D.astype(np.float64), _exact(A, B))


def test_scan_pattern_sums_are_exact():
    """Each row: 8 motif positions, one of 4 base slots set per position (the one-hot
    entries of a k-step); B: E4M3 codes over the whole range (2^-9 .. 448), both signs."""
    rng = np.random.default_rng(2)
    A = np.zeros((128, 32), dtype=np.uint8)
    for r in range(128):
        A[r, 4 * np.arange(8) + rng.integers(0, 4, size=8)] = ONE
    worst = 0.0
    for trial in range(4):
        B = _finite_codes(rng, 32 * 32).reshape(32, 32)
        D = _run(A, B).astype(np.float64)
        want = _exact(A, B)
        worst = max(worst, float(np.max(np.abs(D - want))))
    print("scan-pattern max |error|:", worst)
    assert worst == 0.0


def test_wide_binade_sums_are_exact():
    """32 ones against one large entry and small ones (448 and 31 subnormals down to 2^-9):
    exact sums need 18 significant bits, which FP32 holds; the tensor cores keep them all."""
    rng = np.random.default_rng(3)
    A = np.full((128, 32), ONE, dtype=np.uint8)
    B = np.zeros((32, 32), dtype=np.uint8)
    big = [0x7E, 0x70, 0x60, 0x50]  # 448, 128, 32, 8
    for c in range(32):
        B[c, 0] = big[c % 4]
        B[c, 1:] = rng.integers(0x01, 0x10, size=31)  # subnormals and the smallest normals
    D = _run(A, B).astype(np.float64)
    want = _exact(A, B)
    err = np.abs(D - want)
    rel = err / np.abs(E4M3[B[:, 0]])[None, :]
    print("wide-binade max |error|:", float(err.max()), "relative to the largest term:", float(rel.max()))
    assert float(err.max()) == 0.0
