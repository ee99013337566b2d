"""GPU parity on the shapes of the benchmark's cases, beyond the small random banks.

* a stream like the 1 Gbp precision case (2nd-order Markov background, GC 0.41, 1 % of
  the bases in N runs, motifs of length 5-30, thresholds for p = 1e-4 and 1e-5 from the
  theoretical histograms), 1.2 Mbp of it, every tensor-core mode against the oracle;
* the shards of one stream (equal ranges of window starts plus a halo of the longest
  motif - 1) scanned by the library: their union is the whole stream's hit set;
* blamm_filter_score, the drop-in for the reference's kernel_wrapper, against a
  restatement of filterScore (src/kernel.cu:21-34).

Every comparison is bit-exact: the same (position, column) set and the same score bits.
"""
import numpy as np
import pytest

import oracle
from bankutil import make_bank, make_stream, same_hits
from blamm_gb300 import HIT_DTYPE, GpuScanner, workloads
from blamm_gb300.shard import shard

pytestmark = pytest.mark.gpu


def _markov_case(seed: int, n: int, nmotifs: int):
    rng = np.random.default_rng(seed)
    seqs = []
    left, i = n, 0
    while left > 0:  # a few sequences, each with its N runs
        L = min(left, int(rng.integers(200_000, 500_000)))
        s = workloads.markov2_bases(rng, L, 0.41)
        seqs.append((f"chr{i}", workloads.insert_n_runs(rng, s, 0.01)))
        left -= L
        i += 1
    bases, runs, _, _ = workloads.filtered_stream(seqs)
    pfms = [p for _, p in workloads.random_pfms(rng, nmotifs, 5, 30)]
    counts = np.array([np.count_nonzero((bases | 0x20) == ord(c)) for c in "acgt"], dtype=np.uint64)
    P, lens, thr, _, _ = oracle.motif_bank(pfms, counts, 0.25, (1e-4, 1e-5))
    return bases, runs, P, lens, thr


@pytest.fixture(scope="module")
def markov_case():
    return _markov_case(31, 1_200_000, 120)


@pytest.mark.parametrize("mode", ["auto", "bf16", "bf16x2", "e4m3"])
@pytest.mark.parametrize("pi", [0, 1])
def test_markov_n_runs_stream_matches_oracle(markov_case, mode, pi):
    bases, runs, P, lens, thr = markov_case
    assert len(runs) > 10  # the N runs split the stream
    sc = GpuScanner(0, mode)
    try:
        sc.set_motifs(P, lens, thr[pi])
        got = sc.scan(bases, runs)
        want = oracle.scan(bases, runs, P, lens, thr[pi])
        ok, msg = same_hits(got, want)
        assert ok, msg
        assert len(want) > (2000 if pi == 0 else 200)
    finally:
        sc.close()


@pytest.mark.parametrize("world", [2, 3])
def test_shards_scanned_by_the_library_equal_the_whole_stream(world):
    torch = pytest.importorskip("torch")
    P, lens, thr = make_bank(43, 48, 5, 30, rel=0.86)
    bases, runs = make_stream(44, 900_000, nruns=23, lower_frac=0.02)
    sc = GpuScanner(0, "auto")
    try:
        sc.set_motifs(P, lens, thr)
        whole = sc.scan(bases, runs)
        parts = []
        for r in range(world):
            b, rr, off, keep = shard(bases, runs, r, world, int(lens.max()) - 1)
            d_b = torch.from_numpy(np.ascontiguousarray(b)).cuda()
            d_r = torch.from_numpy(rr).cuda()
            cap = len(whole) + 1024
            d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
            nh = sc.scan_device(d_b.data_ptr(), len(b), d_r.data_ptr(), len(rr), d_h.data_ptr(), cap)
            h = d_h[: nh * HIT_DTYPE.itemsize].cpu().numpy().view(HIT_DTYPE).copy()
            h = h[h["pos"] < keep]
            h["pos"] += off
            parts.append(h)
        ok, msg = same_hits(np.concatenate(parts), whole)
        assert ok, msg
        ok, msg = same_hits(whole, oracle.scan(bases, runs, P, lens, thr))
        assert ok, msg
    finally:
        sc.close()


def _filter_score_ref(R: np.ndarray, m: int, n: int, thr: np.ndarray):
    """filterScore (src/kernel.cu:21-34): every column-major index idx = j*m + i with
    R[idx] >= threshold[j] is appended (in any order) with its value."""
    j = np.arange(m * n) // m
    keep = R >= thr[j]
    return np.flatnonzero(keep).astype(np.int32), R[keep]


@pytest.mark.parametrize("m,n", [(1000, 64), (999, 37), (33, 1), (1, 5)])
def test_filter_score_matches_filterScore(m, n):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(m * 7 + n)
    R = rng.normal(0.0, 3.0, size=m * n).astype(np.float32)
    thr = rng.normal(4.0, 1.0, size=n).astype(np.float32)
    sc = GpuScanner(0, "auto")
    try:
        d_R = torch.from_numpy(R).cuda()
        d_t = torch.from_numpy(thr).cuda()
        # the reference's buffers: 2 * m * n entries (src/pwmscan.cpp:346-352); a first call,
        # then a second one appending onto the first's count
        d_idx = torch.full((2 * m * n,), -1, dtype=torch.int32, device="cuda")
        d_sc = torch.zeros(2 * m * n, dtype=torch.float32, device="cuda")
        d_n = torch.zeros(1, dtype=torch.int32, device="cuda")
        want_i, want_s = _filter_score_ref(R, m, n, thr)
        for call in range(2):
            sc.filter_score(d_R.data_ptr(), m, n, d_t.data_ptr(), d_idx.data_ptr(), d_sc.data_ptr(),
                            d_n.data_ptr())
            torch.cuda.synchronize()
            k = int(d_n.item())
            assert k == (call + 1) * len(want_i)
            got_i = d_idx[call * len(want_i):k].cpu().numpy()
            got_s = d_sc[call * len(want_i):k].cpu().numpy()
            order = np.argsort(got_i, kind="stable")
            assert np.array_equal(got_i[order], want_i)
            assert np.array_equal(got_s[order].view(np.uint32), want_s.view(np.uint32))
        assert len(want_i) > 0 or m * n < 64
    finally:
        sc.close()
