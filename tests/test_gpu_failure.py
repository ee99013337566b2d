"""GPU failure path without a GPU fault: a wait that runs out.

With the stall hook the scan kernel's MMA warp waits on an mbarrier that nothing
completes; the bounded wait gives up after a short limit, every role of every CTA
leaves its loop, outstanding copies and MMAs are drained, tensor memory is freed, and
the call reports BLAMM_ERR_TIMEOUT.  The same context then scans correctly.
"""
import pytest

import oracle
from bankutil import make_bank, make_stream, same_hits
from blamm_gb300 import BlammError
from blamm_gb300._native import BLAMM_ERR_TIMEOUT

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["bf16x2", "bf16", "e4m3"])
def test_a_wait_that_runs_out_reports_timeout_and_the_context_stays_usable(scanner, mode):
    P, lens, thr = make_bank(81, 48, 5, 30, rel=0.85)
    bases, runs = make_stream(82, 400_000, nruns=5)
    scanner.set_mode(mode)
    scanner.set_motifs(P, lens, thr)
    scanner.debug_stall(True, 2_000_000)  # about a millisecond of SM cycles
    try:
        with pytest.raises(BlammError) as e:
            scanner.scan(bases, runs)
        assert e.value.code == BLAMM_ERR_TIMEOUT
    finally:
        scanner.debug_stall(False)
    ok, msg = same_hits(scanner.scan(bases, runs), oracle.scan(bases, runs, P, lens, thr))
    assert ok, msg
