"""GPU theoretical histograms and p-value thresholds (blamm_theoretical_hist).

Pinned two ways: the counts equal the reference's own hist_*.dat files of the
two-sequence golden case, and, on random banks, the oracle's restatement of the
DP; the thresholds equal the host library's (whose CLI output matches the
reference's files) bit for bit.  The FP64 DP variant is checked for closeness.
"""
import os

import numpy as np
import pytest

import oracle
from blamm_gb300 import workloads
from blamm_gb300._native import MotifBank

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "two_sequences_1mbp")


def _bg_prob(counts, pseudo=0.25):
    """Species::getNuclProbabilities (src/species.cpp:63-71) in float32."""
    c = np.asarray(counts, dtype=np.uint64)
    tot = np.float32(c.sum()) + np.float32(4.0) * np.float32(pseudo)
    return ((c.astype(np.float32) + np.float32(pseudo)) / tot).astype(np.float32)


def test_counts_equal_the_reference_hist_files(scanner):
    with open(os.path.join(GOLDEN, "expected", "sequences.mf.dict")) as f:  # the case's dictionary
        counts = [int(x) for x in next(ln for ln in f if ln.startswith("NUCL_COUNT_ACGT")).split()[1:5]]
    bank = MotifBank.load(os.path.join(GOLDEN, "motifs.jaspar"), permutations=True, revcompl=False)
    bank.generate(np.array(counts, dtype=np.uint64), 0.25)
    P, lens, _ = bank.matrix()
    _, cnt = scanner.theoretical_hist(P, lens, _bg_prob(counts), nbins=250, counts=True)
    for c in range(len(lens)):
        path = os.path.join(GOLDEN, "expected", f"hist_cfg1_{bank.name(c)}.dat")
        rows = open(path).read().split("\n")
        want = np.array([int(r.split("\t")[1]) for r in rows[1:] if r.strip()], dtype=np.uint64)
        assert np.array_equal(cnt[c], want), bank.name(c)


@pytest.mark.parametrize("seed", [0, 1])
def test_thresholds_equal_the_host_library(scanner, seed):
    rng = np.random.default_rng(seed)
    pfms = [p for _, p in workloads.random_pfms(rng, 300, 5, 30)]
    counts = np.array([2900, 2100, 2100, 2900], dtype=np.uint64)
    bank = MotifBank.from_pfms(pfms, revcompl=True)
    bank.generate(counts, 0.25)
    P, lens, _ = bank.matrix()
    bgp = _bg_prob(counts)
    pvals = (1e-3, 1e-4, 1e-5)
    thr, cnt = scanner.theoretical_hist(P, lens, bgp, pvals, hist_of=bank.hist_columns(), counts=True)
    for v, pv in enumerate(pvals):
        want = bank.pvalue_thresholds(bgp, pv)
        assert np.array_equal(thr[v].view(np.uint32), want.view(np.uint32)), f"p={pv}"
    # counts of the forward columns against the oracle's DP
    for c in range(0, len(lens), 17):
        h = bank.hist_columns()[c]
        pwm = P[h, :4 * lens[h]].reshape(-1, 4)
        assert np.array_equal(cnt[c], oracle.theoretical_hist(pwm, bgp, 250, 10_000_000)), c


def test_fp64_dp_is_close(scanner):
    rng = np.random.default_rng(5)
    pfms = [p for _, p in workloads.random_pfms(rng, 64, 5, 30)]
    counts = np.array([2500, 2500, 2500, 2500], dtype=np.uint64)
    bank = MotifBank.from_pfms(pfms, revcompl=False)
    bank.generate(counts, 0.25)
    P, lens, _ = bank.matrix()
    bgp = _bg_prob(counts)
    t32, _ = scanner.theoretical_hist(P, lens, bgp, (1e-4,))
    t64, _ = scanner.theoretical_hist(P, lens, bgp, (1e-4,), fp64_dp=True)
    mn, mx = bank.min_max()
    width = (mx - mn) / 250
    assert np.all(np.abs(t64[0] - t32[0]) <= width + 1e-6)
