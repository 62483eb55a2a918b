"""Served form on the GPU: every answer equals the summary of the plain
drop-in call for that query, whether the query runs alone or in a mix of
concurrent BFS and SSSP queries that join and leave the 64 lanes."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(ig, gpu):
    g = ig.rmat(14, 16, seed=17, maxw=1000)
    d = ig.DeviceCSR(g)
    srv = ig.Server(d, max_pending=1024)
    yield g, d, srv
    srv.close()
    d.close()


def plain_answer(ig, g, d, kind, src, targets):
    dist = np.empty(g.nodes, np.int32)
    (ig.GPUbfs_vertex if kind == 0 else ig.GPUsssp_vertex)(int(src), d, dist)
    return ig.summarize(kind, src, dist, targets)


def test_single_queries(ig, served):
    g, d, srv = served
    rng = np.random.default_rng(1)
    for kind in (0, 1):
        for src in [int(x) for x in g.pick_sources(3, seed=11)] + [int(np.argmin(g.degree()))]:
            tg = rng.integers(0, g.nodes, 5)
            a = srv.wait(srv.submit(kind, src, tg))
            assert a.key() == plain_answer(ig, g, d, kind, src, tg).key()


def test_mix_matches_alone(ig, served):
    """200 queries from 4 client threads with staggered arrivals; each answer
    equals the plain call's, so it is also what the query gives alone."""
    g, d, srv = served
    rng = np.random.default_rng(7)
    srcs = g.pick_sources(100, seed=5)
    jobs = [(int(k), int(s), rng.integers(0, g.nodes, 4)) for k in (0, 1) for s in srcs]
    rng.shuffle(jobs)
    answers = {}

    def client(part):
        for i in part:
            kind, s, tg = jobs[i]
            t = srv.submit(kind, s, tg)
            time.sleep(0.0002 * (i % 3))
            answers[i] = t

    threads = [threading.Thread(target=client, args=(range(k, len(jobs), 4),)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    got = {i: srv.wait(t) for i, t in answers.items()}
    for i, (kind, s, tg) in enumerate(jobs):
        assert got[i].key() == plain_answer(ig, g, d, kind, s, tg).key(), (kind, s)
    done, steps = srv.stats()
    assert done >= len(jobs) and steps > 0


def test_busy_when_queue_full(ig, gpu):
    g = ig.rmat(12, 8, seed=3, maxw=100)
    with ig.DeviceCSR(g) as d:
        srv = ig.Server(d, max_pending=2)
        tickets, busy = [], 0
        for i in range(200):
            t = srv.try_submit(0, int(i % g.nodes))
            if t is None:
                busy += 1
            else:
                tickets.append(t)
        for t in tickets:
            srv.wait(t)
        srv.close()
    assert busy > 0 and tickets


def test_bad_queries_rejected(ig, served):
    g, d, srv = served
    with pytest.raises(ig.IndigoError):
        srv.submit(0, g.nodes)
    with pytest.raises(ig.IndigoError):
        srv.submit(2, 0)
    with pytest.raises(ig.IndigoError):
        srv.submit(0, 0, list(range(17)))


def test_memory_admission_defers_then_serves(ig, orc, gpu):
    """With a budget that holds only one engine, BFS and SSSP queries submitted
    together cannot all be admitted at once: queries of the kind without an
    engine are deferred (counted), not failed, until the resident engine
    falls idle and is released; every answer still equals the oracle's."""
    g = ig.rmat(13, 16, seed=19, maxw=1000)
    with ig.DeviceCSR(g) as d:
        srv = ig.Server(d, max_pending=256)
        try:
            srv.wait(srv.submit(1, 0))  # the SSSP engine, the larger one, is resident now
            held_sssp, _, created0 = srv.memory()
            assert held_sssp > 0 and created0 == 1
            srv.set_memory_budget(held_sssp + 1024)  # room for one engine, not both
            rng = np.random.default_rng(5)
            srcs = [int(s) for s in g.pick_sources(24, seed=9)]
            jobs = [(k, s, rng.integers(0, g.nodes, 3)) for s in srcs for k in (0, 1)]
            tickets = [srv.submit(k, s, tg) for k, s, tg in jobs]
            answers = [srv.wait(t, 120000) for t in tickets]
            held, deferred, created = srv.memory()
        finally:
            srv.close()
    assert deferred > 0 and created >= 2  # the SSSP engine released for the BFS engine
    assert held <= held_sssp + 1024
    for (k, s, tg), a in zip(jobs, answers):
        dist = orc.bfs(g, s) if k == 0 else orc.sssp(g, s)
        assert a.key() == ig.summarize(k, s, dist, tg).key(), (k, s)


def test_memory_admission_fails_what_never_fits(ig, gpu):
    """A budget below the SSSP engine's size: SSSP queries complete with
    IG_ERR_NOMEM (they can never be admitted), BFS queries are served."""
    g = ig.rmat(12, 16, seed=3, maxw=100)
    with ig.DeviceCSR(g) as d:
        srv = ig.Server(d, max_pending=64)
        try:
            srv.wait(srv.submit(0, 1))
            held_bfs, _, _ = srv.memory()
            srv.set_memory_budget(held_bfs + (held_bfs >> 2))
            t_s = srv.submit(1, 1)
            with pytest.raises(ig.IndigoError) as e:
                srv.wait(t_s, 60000)
            assert e.value.status == ig._lib.IG_ERR_NOMEM
            assert srv.wait(srv.submit(0, 2), 60000).reached > 0
        finally:
            srv.close()
