"""Multi-rank host logic on the CPU (gloo, world size 2): the bench's
max/sum reductions over ranks, and the edge-balanced split of a batch of
graphs over ranks (every graph on exactly one rank, each rank's slice equal to
the graphs it replaces, work balanced).  No GPU and no device memory."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path[:0] = [str(ROOT), str(ROOT / "parallelization-artifact-sc23_gb300")]
    try:
        import bench
        import indigo_gb300 as ig
        d = bench.Dist()
        mx, sm = d.max(float(rank + 1)), d.sum(float(rank + 1))
        u, vptr = ig.gen_batch(40, vmin=64, vmax=2048, seed=13)
        g0, g1 = ig.split_batch(u, vptr, world)[rank]
        su, sv = ig.take_batch(u, vptr, g0, g1)
        same = all(np.array_equal(ig.unpack(su, sv, i - g0).nlist, ig.unpack(u, vptr, i).nlist) and
                   np.array_equal(ig.unpack(su, sv, i - g0).nindex, ig.unpack(u, vptr, i).nindex)
                   for i in range(g0, g1))
        graphs_all = d.sum(float(g1 - g0))
        edges_all = d.sum(float(su.edges))
        d.barrier()
        d.close()
        out.put((rank, mx, sm, g0, g1, same, graphs_all, edges_all, u.edges))
    except Exception as e:  # reported to the parent
        out.put((rank, repr(e)))


@pytest.mark.timeout(300)
def test_two_ranks_reduce_and_split():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    res = {r[0]: r for r in res}
    for r in (0, 1):
        assert len(res[r]) > 2, res[r]
        _, mx, sm, g0, g1, same, graphs_all, edges_all, e_union = res[r]
        assert mx == 2.0 and sm == 3.0
        assert same
        assert graphs_all == 40 and edges_all == e_union
    assert res[0][3] == 0 and res[0][4] == res[1][3] and res[1][4] == 40


def test_split_balances_edges(ig):
    u, vptr = ig.gen_batch(200, vmin=64, vmax=4096, seed=5)
    eptr = u.nindex.astype(np.int64)[vptr]
    work = np.diff(eptr) + np.diff(vptr.astype(np.int64))
    for parts in (1, 2, 3, 8):
        ranges = ig.split_batch(u, vptr, parts)
        assert ranges[0][0] == 0 and ranges[-1][1] == 200
        assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
        loads = [int(work[a:b].sum()) for a, b in ranges]
        assert max(loads) - min(loads) <= 2 * int(work.max())
    with pytest.raises(ValueError):
        ig.split_batch(u, vptr, 0)


def test_take_whole_batch_is_identity(ig):
    u, vptr = ig.gen_batch(12, vmin=64, vmax=512, seed=3)
    t, tv = ig.take_batch(u, vptr, 0, 12)
    assert t.digest() == u.digest() and np.array_equal(tv, vptr)
