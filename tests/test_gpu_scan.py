"""GPU parity: the fused scan (every mode) against the oracle's sequential-FP32 scan.

Bit-exact: the hit set (position, column) and every score's bits must equal the
oracle's, which restates the reference's BLAS path (pinned in test_oracle_pin.py).
"""
import numpy as np
import pytest

import oracle
from bankutil import exact_window_scores, make_bank, make_stream, quantized_columns, same_hits

pytestmark = pytest.mark.gpu

MODES = ["bf16x2", "bf16", "e4m3", "fp32"]
TERMS = {"bf16x2": 2, "bf16": 1, "e4m3": 8}


@pytest.mark.parametrize("mode", ["bf16x2", "bf16", "e4m3"])
def test_tensor_core_sums_are_exact(scanner, mode):
    """The raw accumulator equals the exact sum of the fixed-point BF16 terms (no rounding)."""
    P, lens, thr = make_bank(1, 40, 5, 30)
    bases, _ = make_stream(2, 5000, lower_frac=0.05)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    p0, npos = 100, 700
    D = scanner.debug_scores(bases, p0, npos)
    Q = quantized_columns(P, lens, TERMS[mode])
    want = exact_window_scores(bases, Q, lens, p0, npos)
    assert np.all(np.float64(np.float32(want)) == want)  # representable
    bad = np.flatnonzero(D.astype(np.float64).ravel() != want.ravel())
    assert bad.size == 0, f"{bad.size} mismatches, first {D.ravel()[bad[0]]} vs {want.ravel()[bad[0]]}"


@pytest.mark.parametrize("mode", ["bf16x2", "bf16", "e4m3"])
@pytest.mark.parametrize("lengths", [(1, 2), (3, 4), (5, 6), (7, 8), (1, 10), (13, 14), (29, 30)])
def test_bias_in_the_last_k_step(scanner, mode, lengths):
    """A tile whose longest motif has length 4g-3 or 4g-2 carries the threshold bias in the
    second K core of its last k-step (no bias MMA); (3, 4), (7, 8) keep the bias MMA. Both
    give the exact sums and the oracle's hits, with some thresholds below every score."""
    lo, hi = lengths
    P, lens, thr = make_bank(100 + lo, 24, lo, hi, rel=0.9)
    thr[::5] = np.float32(-1e3)  # every window of those columns is a hit
    bases, runs = make_stream(200 + lo, 8000, nruns=3, lower_frac=0.05)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    p0, npos = 40, 600
    D = scanner.debug_scores(bases, p0, npos)
    Q = quantized_columns(P, lens, TERMS[mode])
    want = exact_window_scores(bases, Q, lens, p0, npos)
    bad = np.flatnonzero(D.astype(np.float64).ravel() != want.ravel())
    assert bad.size == 0, f"{bad.size} mismatches, first {D.ravel()[bad[0]]} vs {want.ravel()[bad[0]]}"
    got = scanner.scan(bases, runs, hit_cap=None)
    ok, msg = same_hits(got, oracle.scan(bases, runs, P, lens, thr))
    assert ok, msg


@pytest.mark.parametrize("mode", MODES)
def test_scan_matches_oracle(scanner, mode):
    P, lens, thr = make_bank(3, 64, 5, 30, rel=0.88)
    bases, runs = make_stream(4, 300_000, nruns=40, lower_frac=0.02)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    got = scanner.scan(bases, runs)
    want = oracle.scan(bases, runs, P, lens, thr)
    ok, msg = same_hits(got, want)
    assert ok, msg
    assert len(want) > 1000


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("n", [1, 7, 127, 128, 129, 1000, 4099])
def test_small_and_ragged_streams(scanner, mode, n):
    P, lens, thr = make_bank(5, 12, 3, 20, rel=0.6)
    bases, runs = make_stream(6 + n, n, nruns=min(n, 5), lower_frac=0.1)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    ok, msg = same_hits(scanner.scan(bases, runs), oracle.scan(bases, runs, P, lens, thr))
    assert ok, msg


@pytest.mark.parametrize("mode", MODES)
def test_long_motifs_and_single_column(scanner, mode):
    P, lens, thr = make_bank(7, 3, 60, 120, rc=False, rel=0.55)
    bases, runs = make_stream(8, 20_000, nruns=3)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    if mode == "e4m3":  # the E4M3 form takes motifs up to 64 positions
        from blamm_gb300 import BlammError
        with pytest.raises(BlammError):
            scanner.scan(bases, runs)
        return
    ok, msg = same_hits(scanner.scan(bases, runs), oracle.scan(bases, runs, P, lens, thr))
    assert ok, msg
    P1, l1, t1 = P[:1], lens[:1], thr[:1]
    scanner.set_motifs(P1, l1, t1)
    ok, msg = same_hits(scanner.scan(bases, runs), oracle.scan(bases, runs, P1, l1, t1))
    assert ok, msg


@pytest.mark.parametrize("mode", MODES)
def test_many_columns_many_tiles(scanner, mode):
    P, lens, thr = make_bank(9, 700, 5, 30, rel=0.9)
    bases, runs = make_stream(10, 60_000, nruns=10)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    ok, msg = same_hits(scanner.scan(bases, runs), oracle.scan(bases, runs, P, lens, thr))
    assert ok, msg


def test_threshold_update_and_overflow_retry(scanner):
    P, lens, thr = make_bank(11, 20, 6, 16, rel=0.9)
    bases, runs = make_stream(12, 50_000, nruns=4)
    scanner.set_mode("bf16x2")
    scanner.set_motifs(P, lens, thr)
    a = scanner.scan(bases, runs)
    low = thr - np.float32(4.0)
    scanner.set_thresholds(low)
    b = scanner.scan(bases, runs, hit_cap=None)
    ok, msg = same_hits(b, oracle.scan(bases, runs, P, lens, low))
    assert ok, msg
    assert len(b) > len(a)


def test_guard_band_is_small_for_split(scanner):
    P, lens, thr = make_bank(13, 50, 5, 30)
    scanner.set_motifs(P, lens, thr)
    scanner.set_mode("bf16x2")
    g2 = scanner.guard_band()
    scanner.set_mode("bf16")
    g1 = scanner.guard_band()
    assert np.all(g2 > 0) and np.all(g2 < 0.02)
    assert np.all(g1 > g2)
