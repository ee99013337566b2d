"""Multi-GPU path on CPU: gloo ranks scan their own shards (equal ranges of window starts
plus a halo of the longest motif - 1); the gathered hits equal the whole stream's (no
data-path collective, only the final gather)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from blamm_gb300.shard import shard, shard_bounds


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path[:0] = [os.path.dirname(here), os.path.join(os.path.dirname(here), "oracle"), here]
    import oracle
    from bankutil import make_bank, make_stream
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    P, lens, thr = make_bank(41, 24, 5, 20, rel=0.85)
    bases, runs = make_stream(42, 250_000, nruns=17, lower_frac=0.02)
    b, r, off, keep = shard(bases, runs, rank, world, int(lens.max()) - 1)
    h = oracle.scan(b, r, P, lens, thr, nthreads=2)
    h = h[h["pos"] < keep]  # windows starting in the halo belong to the next rank
    mine = [(int(p) + off, int(c), int(s)) for p, c, s in zip(h["pos"], h["col"], h["score"].view(np.uint32))]
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        full = oracle.scan(bases, runs, P, lens, thr, nthreads=2)
        want = sorted((int(p), int(c), int(s)) for p, c, s in zip(full["pos"], full["col"],
                                                                   full["score"].view(np.uint32)))
        got = sorted(x for part in gathered for x in part)
        q.put((got == want, len(want), [len(p) for p in gathered]))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_sharded_scan_equals_whole(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    ok, n, parts = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ok and n > 100 and all(x > 0 for x in parts)


def test_shard_bounds_balance_and_cover():
    for n, world in ((2000, 3), (5, 8), (0, 2), (1_000_000_007, 8)):
        b = shard_bounds(n, world)
        assert len(b) == world and b[0][0] == 0 and b[-1][1] == n
        assert all(b[i][1] == b[i + 1][0] for i in range(world - 1))
        sizes = [hi - lo for lo, hi in b]
        assert max(sizes) - min(sizes) <= 1


def test_shard_run_tables_and_halo():
    runs = np.array([0, 10, 500, 900, 1500], dtype=np.int64)
    bases = np.zeros(2000, dtype=np.uint8)
    b = shard_bounds(2000, 3)
    for r in range(3):
        sb, sr, off, keep = shard(bases, runs, r, 3, 29)
        lo, hi = b[r]
        assert off == lo and keep == hi - lo and len(sb) == min(2000, hi + 29) - lo
        # the run holding lo starts the table; then every run start inside the shard
        want = np.concatenate([[0], runs[(runs > lo) & (runs < lo + len(sb))] - lo])
        assert np.array_equal(sr, want)
    # more ranks than bases: empty shards scan nothing
    assert shard_bounds(2, 4) == [(0, 0), (0, 1), (1, 1), (1, 2)]
    sb, sr, off, keep = shard(bases[:2], runs[:1], 2, 4, 5)
    assert len(sb) == 0 and len(sr) == 0 and keep == 0


def test_one_long_run_splits_evenly_with_a_halo():
    """A stream that is a single run (one chromosome) splits into equal shards, and the
    union of the shards' kept hits is the whole stream's hit set (oracle, in-process)."""
    import oracle
    from bankutil import make_bank, make_stream, same_hits
    P, lens, thr = make_bank(43, 24, 5, 20, rel=0.8)
    bases, _ = make_stream(44, 90_000)
    runs = np.zeros(1, dtype=np.int64)
    want = oracle.scan(bases, runs, P, lens, thr)
    parts = []
    for r in range(3):
        b, rr, off, keep = shard(bases, runs, r, 3, int(lens.max()) - 1)
        assert np.array_equal(rr, [0]) and keep == 30_000 and len(b) == min(90_000, 30_000 * (r + 1) + 19) - off
        h = oracle.scan(b, rr, P, lens, thr)
        h = h[h["pos"] < keep]
        h["pos"] += off
        parts.append(h)
    assert all(len(h) > 0 for h in parts)
    ok, msg = same_hits(np.concatenate(parts), want)
    assert ok, msg
