"""GPU: the scan service (include/blamm_serve.h).

Continuous batching must not change results: every request's hits are the same
(position, column, score bits) alone and in a mix of concurrent requests with
different lengths, column subsets and threshold sets, and equal to the oracle's.
"""
import numpy as np
import pytest

import oracle
from bankutil import make_bank, make_stream, same_hits
from blamm_gb300 import Server

pytestmark = pytest.mark.gpu


def _requests(rng, ncols, k):
    reqs = []
    for i in range(k):
        n = int(np.exp(rng.uniform(np.log(1_000), np.log(400_000))))
        bases, runs = make_stream(500 + i, n, nruns=int(rng.integers(1, 6)), lower_frac=0.01)
        size = int(rng.integers(1, ncols + 1))
        cols = None if rng.random() < 0.15 else np.sort(rng.choice(ncols, size=size, replace=False))
        reqs.append((bases, runs, cols, int(rng.integers(0, 2))))
    return reqs


def test_requests_alone_and_in_the_mix_give_the_same_hits():
    P, lens, thr0 = make_bank(71, 150, 5, 30, rel=0.84)
    thr1 = (thr0 + 0.6).astype(np.float32)  # a second, stricter threshold set
    sets = np.stack([thr0, thr1])
    reqs = _requests(np.random.default_rng(72), len(lens), 24)

    alone = []
    srv = Server(P, lens, sets, slots=1)
    try:
        for bases, runs, cols, st in reqs:
            alone.append(srv.take(srv.submit(bases, runs, cols, st)))
    finally:
        srv.close()

    srv = Server(P, lens, sets, slots=4)
    try:
        ids = [srv.submit(b, r, c, s) for b, r, c, s in reqs]  # all queued at once
        mixed = [srv.take(i) for i in ids]
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
    finally:
        srv.close()

    for k, ((bases, runs, cols, s), a, m) in enumerate(zip(reqs, alone, mixed)):
        ok, msg = same_hits(a, m)
        assert ok, f"request {k}: alone vs mix: {msg}"
        if k % 6 == 0:  # the oracle on a few
            sub = np.arange(len(lens)) if cols is None else cols
            t = sets[s]
            want = oracle.scan(bases, runs, P[sub], lens[sub], t[sub])
            want["col"] = sub[want["col"]]
            ok, msg = same_hits(a, want)
            assert ok, f"request {k}: vs oracle: {msg}"


def test_admission_by_memory_budget_serialises_large_requests():
    P, lens, thr = make_bank(73, 40, 5, 20, rel=0.85)
    reqs = _requests(np.random.default_rng(74), len(lens), 6)
    # a budget that admits one request at a time still completes all of them, with the same hits
    srv = Server(P, lens, thr[None, :], slots=3, hbm_budget=96 << 20)
    try:
        ids = [srv.submit(b, r, c, 0) for b, r, c, _ in reqs]
        got = [srv.take(i) for i in ids]
    finally:
        srv.close()
    for (bases, runs, cols, _), g in zip(reqs, got):
        sub = np.arange(len(lens)) if cols is None else cols
        want = oracle.scan(bases, runs, P[sub], lens[sub], thr[sub])
        want["col"] = sub[want["col"]]
        ok, msg = same_hits(g, want)
        assert ok, msg


def test_admission_counts_the_buffers_slots_keep():
    """Slots keep the device buffers of earlier requests; admission counts them, and when the
    queue's head does not fit with nothing in flight the slots release theirs.  A budget a little
    above one request's estimate keeps the committed bytes (requests in flight + kept buffers)
    within it at every admission and completion, and every request still gets its hits."""
    from blamm_gb300 import GpuScanner
    P, lens, thr = make_bank(75, 40, 5, 20, rel=0.85)
    reqs = _requests(np.random.default_rng(76), len(lens), 10)
    sc = GpuScanner(0, "auto")  # how many bytes one slot keeps after a request
    try:
        sc.set_motifs(P, lens, thr)
        b, r, _, _ = max(reqs, key=lambda q: len(q[0]))
        sc.scan(b, r)
        kept = sc.call_bytes()
        assert kept > 0
        sc.release_buffers()
        assert sc.call_bytes() == 0
        ok, msg = same_hits(sc.scan(b, r), oracle.scan(b, r, P, lens, thr))  # usable after the release
        assert ok, msg
    finally:
        sc.close()
    budget = 2 * kept + (24 << 20)
    srv = Server(P, lens, thr[None, :], slots=4, hbm_budget=budget)
    try:
        ids = [srv.submit(b, r, c, 0) for b, r, c, _ in reqs]
        got = [srv.take(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert 0 < st["peak_committed"] <= st["budget"]
    assert st["bytes_held"] <= st["budget"]
    for (bases, runs, cols, _), g in zip(reqs, got):
        sub = np.arange(len(lens)) if cols is None else cols
        want = oracle.scan(bases, runs, P[sub], lens[sub], thr[sub])
        want["col"] = sub[want["col"]]
        ok, msg = same_hits(g, want)
        assert ok, msg
