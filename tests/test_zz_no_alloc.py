"""blamm_scan_device_static (the allocation-free entry point) against blamm_scan_device.

Collected last on purpose (file name): it must give the same hits whether it is the
first scan of the process or runs after every other test.  The comparison is exact:
same (position, column) set and the same score bits.
"""
import numpy as np
import pytest

from bankutil import make_bank, make_stream, same_hits
from blamm_gb300 import HIT_DTYPE, GpuScanner
from blamm_gb300._native import BLAMM_ERR_ARG, BLAMM_ERR_STATE, BlammError

pytestmark = pytest.mark.gpu

STATIC_MAX_BASES = 4 << 20


def _device_case(n: int, seed: int):
    torch = pytest.importorskip("torch")
    P, lens, thr = make_bank(seed, 96, 5, 30, rel=0.92)
    bases, runs = make_stream(seed + 1, n, nruns=17, lower_frac=0.01)
    d_b = torch.from_numpy(bases).cuda()
    d_r = torch.from_numpy(runs).cuda()
    return torch, P, lens, thr, d_b, d_r, len(runs)


def _hits(torch, d_h, nh: int) -> np.ndarray:
    return d_h[: nh * HIT_DTYPE.itemsize].cpu().numpy().view(HIT_DTYPE).copy()


@pytest.mark.parametrize("mode", ["bf16x2", "bf16", "fp32"])
def test_static_matches_scan_device_twice(mode):
    n = 3_000_000
    torch, P, lens, thr, d_b, d_r, nruns = _device_case(n, 11)
    sc = GpuScanner(0, mode)
    try:
        sc.set_motifs(P, lens, thr)
        cap = 4 << 20
        d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        nh = sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), nruns, d_h.data_ptr(), cap)
        want = _hits(torch, d_h, nh)
        assert nh > 1000
        for call in range(2):
            d_h.zero_()
            got_n = sc.scan_device_static(d_b.data_ptr(), n, d_r.data_ptr(), nruns, d_h.data_ptr(), cap)
            ok, msg = same_hits(_hits(torch, d_h, got_n), want)
            assert ok, f"call {call}: {msg}"
    finally:
        sc.close()


def test_static_rejects_oversize_and_missing_plan():
    torch, P, lens, thr, d_b, d_r, nruns = _device_case(4096, 12)
    sc = GpuScanner(0, "bf16x2")
    try:
        sc.set_motifs(P, lens, thr)
        cap = 1 << 16
        d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        # no plan yet for this bank: the entry point refuses instead of allocating one
        with pytest.raises(BlammError) as e:
            sc.scan_device_static(d_b.data_ptr(), 4096, d_r.data_ptr(), nruns, d_h.data_ptr(), cap)
        assert e.value.code == BLAMM_ERR_STATE
        sc.scan_device(d_b.data_ptr(), 4096, d_r.data_ptr(), nruns, d_h.data_ptr(), cap)
        # more positions than the fixed scratch holds: rejected before any launch
        with pytest.raises(BlammError) as e:
            sc.scan_device_static(d_b.data_ptr(), STATIC_MAX_BASES + 1, d_r.data_ptr(), nruns,
                                  d_h.data_ptr(), cap)
        assert e.value.code == BLAMM_ERR_ARG
        assert "static limit" in str(e.value)
    finally:
        sc.close()


def test_static_at_the_position_limit_matches_scan_device():
    """n equal to the fixed scratch's limit (the offsets of its regions are sized for it)."""
    torch = pytest.importorskip("torch")
    n = STATIC_MAX_BASES
    P, lens, thr = make_bank(21, 12, 5, 30, rel=0.93)
    bases, runs = make_stream(22, n, nruns=9, lower_frac=0.01)
    d_b = torch.from_numpy(bases).cuda()
    d_r = torch.from_numpy(runs).cuda()
    sc = GpuScanner(0, "bf16")
    try:
        sc.set_motifs(P, lens, thr)
        cap = 2 << 20
        d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        nh = sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap)
        want = _hits(torch, d_h, nh)
        assert nh > 100
        d_h.zero_()
        got_n = sc.scan_device_static(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap)
        ok, msg = same_hits(_hits(torch, d_h, got_n), want)
        assert ok, msg
    finally:
        sc.close()


def test_static_overflow_returns():
    """More candidate records than the fixed scratch holds, and more hits than the caller's
    buffer: both end in BLAMM_ERR_OVERFLOW; the context then scans normally again."""
    torch = pytest.importorskip("torch")
    from blamm_gb300._native import BLAMM_ERR_OVERFLOW
    n = 3_000_000
    P, lens, thr = make_bank(23, 48, 5, 12, rel=0.3)  # most windows pass: ~n x 3 records
    bases, runs = make_stream(24, n, nruns=5)
    d_b = torch.from_numpy(bases).cuda()
    d_r = torch.from_numpy(runs).cuda()
    sc = GpuScanner(0, "bf16")
    try:
        sc.set_motifs(P, lens, thr)
        cap = 1 << 16
        d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        sc.scan_device(d_b.data_ptr(), 4096, d_r.data_ptr(), 1, d_h.data_ptr(), cap, overflow_ok=True)  # plan
        with pytest.raises(BlammError) as e:
            sc.scan_device_static(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap)
        assert e.value.code == BLAMM_ERR_OVERFLOW and "static limit" in str(e.value)
        # hits beyond the caller's capacity (a stream short enough for the records)
        m = 40_000
        with pytest.raises(BlammError) as e:
            sc.scan_device_static(d_b.data_ptr(), m, d_r.data_ptr(), 1, d_h.data_ptr(), 16)
        assert e.value.code == BLAMM_ERR_OVERFLOW
        # the context and the scratch are still good
        P2, l2, t2 = make_bank(25, 24, 5, 20, rel=0.9)
        sc.set_motifs(P2, l2, t2)
        nh = sc.scan_device(d_b.data_ptr(), m, d_r.data_ptr(), 1, d_h.data_ptr(), cap)
        want = _hits(torch, d_h, nh)
        d_h.zero_()
        got = sc.scan_device_static(d_b.data_ptr(), m, d_r.data_ptr(), 1, d_h.data_ptr(), cap)
        ok, msg = same_hits(_hits(torch, d_h, got), want)
        assert ok, msg
    finally:
        sc.close()
