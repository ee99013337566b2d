"""GPU: column subsets, enqueued and graph-captured scans, the autotuner, and batching.

Every comparison is exact (same (position, column) set, same score bits), against the
oracle or against the synchronous blamm_scan_device.
"""
import numpy as np
import pytest

import oracle
from bankutil import make_bank, make_stream, same_hits
from blamm_gb300 import HIT_DTYPE

pytestmark = pytest.mark.gpu

MODES = ["bf16x2", "bf16", "e4m3", "fp32"]


def _torch():
    return pytest.importorskip("torch")


def _hits(d_h, nh: int) -> np.ndarray:
    return d_h[: nh * HIT_DTYPE.itemsize].cpu().numpy().view(HIT_DTYPE).copy()


@pytest.mark.parametrize("mode", MODES)
def test_column_subset_matches_oracle(scanner, mode):
    P, lens, thr = make_bank(31, 80, 5, 30, rel=0.82)
    bases, runs = make_stream(32, 300_000, nruns=9, lower_frac=0.02)
    rng = np.random.default_rng(33)
    sub = np.sort(rng.choice(len(lens), size=37, replace=False)).astype(np.int32)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    scanner.set_columns(sub[::-1].copy())  # order of the list does not matter
    got = scanner.scan(bases, runs)
    want = oracle.scan(bases, runs, P[sub], lens[sub], thr[sub])
    want["col"] = sub[want["col"]]
    ok, msg = same_hits(got, want)
    assert ok, msg
    # back to the whole bank
    scanner.set_columns(None)
    ok, msg = same_hits(scanner.scan(bases, runs), oracle.scan(bases, runs, P, lens, thr))
    assert ok, msg


def test_column_subset_rejects_bad_lists(scanner):
    from blamm_gb300 import BlammError
    P, lens, thr = make_bank(34, 8, 5, 12)
    scanner.set_mode("bf16x2")
    scanner.set_motifs(P, lens, thr)
    with pytest.raises(BlammError):
        scanner.set_columns([0, 3, 3])
    with pytest.raises(BlammError):
        scanner.set_columns([0, len(lens)])
    scanner.set_columns(None)


@pytest.mark.parametrize("mode", MODES)
def test_enqueue_and_graph_match_scan_device(scanner, mode):
    torch = _torch()
    P, lens, thr = make_bank(41, 64, 5, 30, rel=0.86)
    bases, runs = make_stream(42, 1_500_000, nruns=23, lower_frac=0.01)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    d_b = torch.from_numpy(bases).cuda()
    d_r = torch.from_numpy(runs).cuda()
    cap = 1 << 21
    d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    nh = scanner.scan_device(d_b.data_ptr(), len(bases), d_r.data_ptr(), len(runs), d_h.data_ptr(), cap)
    want = _hits(d_h, nh)
    assert nh > 1000

    scanner.reserve(len(bases), 1 << 22)
    d_c = torch.zeros(4, dtype=torch.int64, device="cuda")
    d_h.zero_()
    scanner.enqueue(d_b.data_ptr(), len(bases), d_r.data_ptr(), len(runs), d_h.data_ptr(), cap, d_c.data_ptr())
    torch.cuda.synchronize()
    c = d_c.cpu().numpy()
    assert c[2] == 0 and c[1] == nh
    ok, msg = same_hits(_hits(d_h, int(c[1])), want)
    assert ok, "enqueue: " + msg

    g = scanner.graph_create(d_b.data_ptr(), len(bases), d_r.data_ptr(), len(runs), d_h.data_ptr(), cap,
                             d_c.data_ptr())
    try:
        for rep in range(2):
            d_h.zero_()
            torch.cuda.synchronize()
            scanner.graph_launch(g)
            torch.cuda.synchronize()
            c = d_c.cpu().numpy()
            assert c[2] == 0 and c[1] == nh, c
            ok, msg = same_hits(_hits(d_h, int(c[1])), want)
            assert ok, f"graph launch {rep}: {msg}"
    finally:
        scanner.graph_destroy(g)


def test_enqueue_needs_a_reservation(scanner):
    torch = _torch()
    from blamm_gb300 import BlammError
    P, lens, thr = make_bank(43, 16, 5, 20)
    scanner.set_mode("bf16x2")
    scanner.set_motifs(P, lens, thr)
    bases, runs = make_stream(44, 50_000)
    d_b = torch.from_numpy(bases).cuda()
    d_r = torch.from_numpy(runs).cuda()
    d_h = torch.empty(1024 * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_c = torch.zeros(4, dtype=torch.int64, device="cuda")
    # a new bank invalidates the plan: enqueue refuses until blamm_reserve rebuilds it
    with pytest.raises(BlammError):
        scanner.enqueue(d_b.data_ptr(), len(bases), d_r.data_ptr(), len(runs), d_h.data_ptr(), 1024,
                        d_c.data_ptr())


def test_autotune_keeps_the_hit_set(scanner):
    torch = _torch()
    P, lens, thr = make_bank(51, 200, 5, 30, rel=0.85)
    bases, runs = make_stream(52, 1_000_000, nruns=5)
    scanner.set_mode("bf16x2")
    scanner.set_motifs(P, lens, thr)
    d_b = torch.from_numpy(bases).cuda()
    d_r = torch.from_numpy(runs).cuda()
    ms = scanner.autotune(d_b.data_ptr(), len(bases), d_r.data_ptr(), len(runs))
    assert ms > 0
    ok, msg = same_hits(scanner.scan(bases, runs), oracle.scan(bases, runs, P, lens, thr))
    assert ok, msg


def test_auto_mode_chooses_a_term_count_and_keeps_the_hit_set():
    """The default mode: one BF16 term until the autotuner has timed one and two terms
    on its sample; either way the hits equal the oracle's."""
    torch = _torch()
    from blamm_gb300 import GpuScanner
    P, lens, thr = make_bank(53, 160, 5, 30, rel=0.85)
    bases, runs = make_stream(54, 1_500_000, nruns=4)
    sc = GpuScanner(0)
    try:
        assert sc.mode == "auto"
        sc.set_motifs(P, lens, thr)
        assert sc.terms() == 1
        want = oracle.scan(bases, runs, P, lens, thr)
        ok, msg = same_hits(sc.scan(bases, runs), want)
        assert ok, msg
        d_b = torch.from_numpy(bases).cuda()
        d_r = torch.from_numpy(runs).cuda()
        assert sc.autotune(d_b.data_ptr(), len(bases), d_r.data_ptr(), len(runs)) > 0
        assert sc.terms() in (1, 2)
        ok, msg = same_hits(sc.scan(bases, runs), want)
        assert ok, msg
        sc.set_mode("fp32")
        assert sc.terms() == 0
    finally:
        sc.close()


def test_many_short_sequences_one_call_equals_one_call_each(scanner):
    """Batching: 600 promoter-like sequences in one stream (one run each) give, per
    sequence, exactly the hits of that sequence scanned alone."""
    rng = np.random.default_rng(61)
    P, lens, thr = make_bank(62, 48, 6, 25, rel=0.84)
    scanner.set_mode("bf16x2")
    scanner.set_motifs(P, lens, thr)
    lengths = np.clip(rng.lognormal(np.log(2000), 1.0, size=600), 200, 50_000).astype(np.int64)
    seqs = [make_stream(1000 + i, int(L))[0] for i, L in enumerate(lengths)]
    starts = np.concatenate([[0], np.cumsum(lengths)[:-1]]).astype(np.int64)
    batch = scanner.scan(np.concatenate(seqs), starts)
    seq_of = np.searchsorted(starts, batch["pos"], side="right") - 1
    for i in range(0, len(seqs), 37):
        alone = scanner.scan(seqs[i], np.zeros(1, dtype=np.int64))
        mine = batch[seq_of == i].copy()
        mine["pos"] -= starts[i]
        ok, msg = same_hits(mine, alone)
        assert ok, f"sequence {i}: {msg}"


@pytest.mark.parametrize("mode", MODES)
def test_pipelined_host_scan_equals_device_scan(mode):
    """blamm_scan on a stream longer than two pipeline chunks (16 Mi positions each, copies on
    a second stream) gives the hit set of one device-resident scan, with runs that start just
    before, at and just after the chunk boundaries and inside the overlap."""
    torch = _torch()
    from blamm_gb300 import GpuScanner
    P, lens, thr = make_bank(71, 48, 5, 30, rel=0.86)
    n = 40_000_000
    bases, runs = make_stream(72, n, nruns=40, lower_frac=0.002)
    chunk = 16 << 20
    extra = [chunk - 3, chunk, chunk + 2, chunk + 17, 2 * chunk - 1, 2 * chunk + 5]
    runs = np.unique(np.concatenate([runs, np.array(extra, dtype=np.int64)]))
    sc = GpuScanner(0, mode)
    try:
        sc.set_motifs(P, lens, thr)
        got = sc.scan(bases, runs)
        d_b = torch.from_numpy(bases).cuda()
        d_r = torch.from_numpy(runs).cuda()
        cap = len(got) + 4096
        d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        nh = sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap)
        want = _hits(d_h, nh)
        assert len(got) > 10_000
        ok, msg = same_hits(got, want)
        assert ok, msg
    finally:
        sc.close()


@pytest.mark.parametrize("mode", ["bf16x2", "bf16"])
def test_role_timing_instance_keeps_the_hit_set(scanner, mode):
    """The role-timing instance of the scan kernel (blamm_debug_profile) finds the same hits
    and fills its counters: every job of every CTA counted once."""
    P, lens, thr = make_bank(91, 64, 5, 30, rel=0.85)
    bases, runs = make_stream(92, 2_000_000, nruns=7)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    want = scanner.scan(bases, runs)
    scanner.profile(True)
    try:
        got = scanner.scan(bases, runs)
        prof = scanner.profile_read()
    finally:
        scanner.profile(False)
    ok, msg = same_hits(got, want)
    assert ok, msg
    st = scanner.stats()
    jobs = st["tiles"] * ((len(bases) + 127) // 128)
    assert 0 < prof.shape[0] <= jobs and int(prof[:, 10].sum()) == jobs
    assert (prof[:, 3] > 0).all()  # the issuers' loop time


@pytest.mark.parametrize("mode", ["bf16x2", "bf16"])
def test_pipelined_scan_with_a_candidate_overflow_falls_back(mode):
    """A permissive bank (3 % of positions x columns are hits) overflows the pipelined path's
    candidate buffer in every chunk: the call falls back to the synchronous chunked path (its
    per-chunk scan timing shows it) and still returns the device-resident scan's hits."""
    torch = _torch()
    from blamm_gb300 import GpuScanner
    P, lens, thr = make_bank(93, 4, 5, 8, rel=0.85)
    n = 34_000_000
    bases, runs = make_stream(94, n, nruns=9)
    sc = GpuScanner(0, mode)
    try:
        sc.set_motifs(P, lens, thr)
        # a fresh context and room for every hit: the first call meets the small candidate buffer
        got = sc.scan(bases, runs, hit_cap=n * len(lens) // 16)
        assert sc.stats()["scan_ms"] > 0  # only the synchronous chunked path times its scans
        d_b = torch.from_numpy(bases).cuda()
        d_r = torch.from_numpy(runs).cuda()
        cap = len(got) + 4096
        d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        nh = sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap)
        assert len(got) > 5_000_000
        ok, msg = same_hits(got, _hits(d_h, nh))
        assert ok, msg
    finally:
        sc.close()
