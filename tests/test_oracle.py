"""The CPU oracle (oracle/indigo_oracle.c) pinned against the reference's own
programs: committed golden fixtures (tests/golden, made by
tests/golden/make_golden.py from oracle/_ref), analytic known answers, and --
when the reference tree is present -- a live run of oracle/_ref."""
import hashlib
import math
import os
import tempfile

import numpy as np
import pytest

from conftest import golden_graphs, kat_graphs


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def graphs(ig):
    return {k: v() for k, v in golden_graphs(ig).items()}


@pytest.mark.parametrize("name", ["grid64", "rmat12", "road64", "er4k", "rmat12_dord"])
def test_oracle_matches_reference_fixtures(orc, golden, graphs, name):
    _, A = golden
    g = graphs[name]
    for k, s in enumerate(A[f"{name}/sources"]):
        assert np.array_equal(orc.bfs(g, int(s)), A[f"{name}/bfs{k}"])
        assert np.array_equal(orc.sssp(g, int(s)), A[f"{name}/sssp{k}"])
    assert np.array_equal(orc.cc(g), A[f"{name}/cc"])
    assert np.array_equal(orc.mis(g), A[f"{name}/mis"])
    assert orc.tc(g) == int(A[f"{name}/tc"][0])
    scores, it, _ = orc.pr_f32(g, 1e-4, 100)
    assert np.array_equal(scores, A[f"{name}/pr"])  # bit-exact FP32 restatement


def test_oracle_grid256_digests(orc, golden, graphs):
    meta, _ = golden
    m = meta["digest_only"]["grid256"]
    g = graphs["grid256"]
    for k, s in enumerate(m["sources"]):
        assert sha(orc.bfs(g, s)) == m["sha256"][f"bfs{k}"]
        assert sha(orc.sssp(g, s)) == m["sha256"][f"sssp{k}"]
    assert sha(orc.cc(g)) == m["sha256"]["cc"]
    mis = orc.mis(g)
    assert sha(mis) == m["sha256"]["mis"] and int((mis == 1).sum()) == 23933
    assert sha(orc.pr_f32(g, 1e-4, 100)[0]) == m["sha256"]["pr"]
    assert orc.tc(g) == 0


def test_known_answers(ig, orc):
    K = kat_graphs(ig)
    n = 256
    g = ig.grid2d(n, n)
    d = orc.bfs(g, 0)
    y, x = np.divmod(np.arange(n * n), n)
    assert np.array_equal(d, x + y)  # Manhattan distance
    assert np.array_equal(orc.bfs(K["path"], 10), np.abs(np.arange(50) - 10))
    k = K["complete"].nodes
    assert orc.tc(K["complete"]) == math.comb(k, 3)
    assert int((orc.mis(K["complete"]) == 1).sum()) == 1
    star = orc.mis(K["star"])
    assert (star[0] == 1 and np.all(star[1:] == 2)) or (star[0] == 2 and np.all(star[1:] == 1))
    lab = orc.cc(K["two_grids"])
    assert set(np.unique(lab).tolist()) == {0, 100}
    assert np.array_equal(orc.bfs(K["single"], 0), [0])
    assert np.array_equal(orc.cc(K["two_isolated"]), [0, 1])
    assert np.array_equal(orc.mis(K["two_isolated"]), [1, 1])


def test_mis_is_greedy_by_unsigned_priority(ig, orc):
    """The reference C++ set equals sequential greedy in decreasing
    (unsigned priority, id) order."""
    g = ig.rmat(11, 8, seed=5)
    st = orc.mis(g)
    pr = np.array([orc.mis_hash(v + 712313887) for v in range(g.nodes)], dtype=np.uint64)
    order = np.lexsort((np.arange(g.nodes), pr))[::-1]
    inset = np.zeros(g.nodes, bool)
    blocked = np.zeros(g.nodes, bool)
    for v in order:
        if not blocked[v]:
            inset[v] = True
            blocked[g.nlist[g.nindex[v]:g.nindex[v + 1]]] = True
    assert np.array_equal(st == 1, inset)


def test_threaded_baselines_agree_with_serial(ig, orc):
    g = ig.rmat(11, 16, seed=9, maxw=1000)
    s = int(g.pick_sources(1, 3)[0])
    assert np.array_equal(orc.bfs_threads(g, s, 4)[0], orc.bfs(g, s))
    assert np.array_equal(orc.sssp_threads(g, s, 4)[0], orc.sssp(g, s))
    assert np.array_equal(orc.cc_threads(g, 4)[0], orc.cc(g))
    st, _ = orc.mis_threads(g, 4)
    assert set(np.unique(st).tolist()) <= {1, 2}
    assert orc.tc_threads(g, 4)[0] == orc.tc(g)
    p4, it4, _ = orc.pr_threads(g, 4, 1e-6, 100)
    p1, it1, _ = orc.pr_f32(g, 1e-6, 100)
    assert abs(it4 - it1) <= 1 and np.abs(p4 - p1).sum() < 1e-5


def test_pr_f64_converges(ig, orc):
    g = ig.rmat(10, 16, seed=3)
    s, it, res = orc.pr_f64(g, epsilon=1e-13, max_iter=2000)
    assert res < 1e-13 and it < 2000


def _reference_sources() -> bool:
    from oracle import oracle
    return oracle.stage_ref()


@pytest.mark.skipif(not _reference_sources(), reason="reference sources neither present nor staged")
def test_oracle_against_live_reference_programs(ig, orc):
    assert orc.build_ref()
    g = ig.rmat(11, 16, seed=21, maxw=1000)
    s = int(g.pick_sources(1, 5)[0])
    with tempfile.TemporaryDirectory() as d:
        egr = os.path.join(d, "g.egr")
        g.write_egr(egr)
        out = os.path.join(d, "o")
        orc.run_ref("bfs", egr, out, 2, s)
        assert np.array_equal(np.fromfile(out, np.int32), orc.bfs(g, s))
        orc.run_ref("sssp", egr, out, 2, s)
        assert np.array_equal(np.fromfile(out, np.int32), orc.sssp(g, s))
        orc.run_ref("cc", egr, out, 2)
        assert np.array_equal(np.fromfile(out, np.int32), orc.cc(g))
        orc.run_ref("mis", egr, out, 2)
        assert np.array_equal(np.fromfile(out, np.uint8), orc.mis(g))
        orc.run_ref("pr", egr, out, 1)
        assert np.array_equal(np.fromfile(out, np.float32), orc.pr_f32(g, 1e-4, 100)[0])
        orc.run_ref("tc", egr, out, 1)
        assert int(np.fromfile(out, np.int64)[0]) == orc.tc(g)


@pytest.mark.skipif(not _reference_sources(), reason="reference sources neither present nor staged")
def test_reference_timing_programs(ig, orc, tmp_path):
    """The CPU arm's timing programs (the reference's best-published
    variants) answer requests with results that agree with the oracle."""
    assert orc.build_ref()
    g = ig.rmat(11, 16, seed=21, maxw=1000)
    gd = g.degree_ordered()
    egr, egr_d = str(tmp_path / "g.egr"), str(tmp_path / "gd.egr")
    g.write_egr(egr)
    gd.write_egr(egr_d)
    srcs = [int(s) for s in g.pick_sources(2, 5)]
    with orc.RefTimer("bfs", egr, 2) as t:
        for s in srcs:
            sec, reached = t.run(s)
            assert sec >= 0 and reached == int((orc.bfs(g, s) != 2147483647).sum())
    with orc.RefTimer("sssp", egr, 2) as t:
        d = orc.sssp(g, srcs[0])
        assert t.run(srcs[0])[1] == int(d[d != 2147483647].astype(np.int64).sum())
    with orc.RefTimer("cc", egr, 2) as t:
        lab = orc.cc(g)
        assert t.run()[1] == int((lab == np.arange(g.nodes)).sum())
    with orc.RefTimer("mis", egr, 2) as t:
        assert t.run()[1] > 0
    with orc.RefTimer("pr", egr, 2) as t:
        assert 0 < t.run()[1] <= 1_000_000_000 + 1000
    with orc.RefTimer("tc", egr_d, 2) as t:
        assert t.run()[1] == orc.tc(gd)
