"""Multi-GPU path on CPU: two gloo ranks scan their own shards; the gathered hits
equal the whole stream's (no data-path collective, only the final gather)."""
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
    b, r, off = shard(bases, runs, rank, world)
    h = oracle.scan(b, r, P, lens, thr, nthreads=2)
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


def test_shard_bounds_cover_stream_at_run_starts():
    runs = np.array([0, 10, 500, 900, 1500], dtype=np.int64)
    b = shard_bounds(2000, runs, 3)
    assert b[0][0] == 0 and b[-1][1] == 2000
    assert all(b[i][1] == b[i + 1][0] for i in range(2))
    assert all(lo in runs or lo == 0 for lo, _ in b)
    bases = np.zeros(2000, dtype=np.uint8)
    for r in range(3):
        sb, sr, off = shard(bases, runs, r, 3)
        assert sr[0] == 0 and off == b[r][0] and len(sb) == b[r][1] - b[r][0]
