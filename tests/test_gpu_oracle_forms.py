"""The batched form, the served form and the edge-centric entry points,
each checked directly against the CPU oracle (not against this library's
plain calls), and PageRank against the converged FP64 oracle.

* Batched: the first 64 graphs of the 4096-graph pack (vertex counts
  log-uniform in [1024, 65536], even graphs Erdos-Renyi with average degree
  8, odd graphs RMAT with edge factor 8, seed 13, weights in [1, 255]);
  ig_gen_batch derives graph i from (seed, i) alone, so these are exactly
  the pack's first 64 graphs.  Per graph: BFS levels from local vertex 0
  (CPUserialDijkstra with unit weights, include/bfs_vertex_cpp.h:52-77), CC
  min-id labels, TC count (h_triCounting, include/tc_vertex_cpp.h:88-107)
  bit-exact; PageRank within 1e-6 relative L1 of the FP64 oracle run for the
  same iteration count.
* Served: RMAT scale 16 (seed 17, weights in [1, 1000]); every BFS / SSSP
  answer (vertices reached, largest and summed distance, target distances)
  equals the summary of the oracle's distance vector (CPUserialDijkstra,
  include/sssp_vertex_cpp.h:88-113), alone and in a mix of queries from
  several client threads.
* Edge forms: GPUbfs_edge, GPUsssp_edge, GPUcc_edge, GPUmis_edge and
  GPUtc_edge through the C ABI, bit-exact against the oracle.
* PageRank: stopping at an L1 residual of 1e-6 leaves a truncation error of
  a few 1e-6 against the converged FP64 solution (L1 residual 1e-12) on
  low-diameter graphs; run to a residual of 1e-7 the FP32 scores are within
  1e-6 relative L1 of it.  Both figures are printed per graph."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PR_TOL = 1e-6  # relative L1 against FP64


# ------------------------------------------------------------------ batched
@pytest.fixture(scope="module")
def pack64(ig, gpu):
    u, vptr = ig.gen_batch(64, vmin=1024, vmax=65536, er_degree=8.0, rmat_edge_factor=8, seed=13, maxw=255)
    return u, vptr


def test_batch_pack_sample_sizes(ig, pack64):
    u, vptr = pack64
    sizes = np.diff(vptr)
    assert sizes.min() >= 1024 and sizes.max() <= 65536
    # log-uniform: both decades of the range are populated
    assert (sizes < 8192).sum() >= 8 and (sizes >= 8192).sum() >= 8


def test_batch_against_oracle(ig, orc, pack64):
    u, vptr = pack64
    G = len(vptr) - 1
    with ig.Batch(u, vptr) as b:
        V = b.nodes
        dist, lab, cnt = ig.DeviceBuffer(4 * V), ig.DeviceBuffer(4 * V), ig.DeviceBuffer(8 * G)
        init = np.concatenate([np.full(int(vptr[i + 1] - vptr[i]), np.float32(1.0) / np.float32(vptr[i + 1] - vptr[i]),
                                       np.float32) for i in range(G)])
        sc = ig.DeviceBuffer.from_array(init)
        its = ig.DeviceBuffer(4 * G)
        for call in range(2):  # direct, then captured into a CUDA graph
            ig.check(ig.load().ig_memcpy(sc.ptr, init.ctypes.data, init.nbytes, 1))
            b.bfs(dist)
            b.cc(lab)
            b.tc(cnt)
            b.pagerank(sc, 1e-6, 100, its)
            assert b.last_run().status == 0
        d, l = dist.to_array(np.int32, V), lab.to_array(np.int32, V)
        c, s, it = cnt.to_array(np.uint64, G), sc.to_array(np.float32, V), its.to_array(np.int32, G)
    worst = 0.0
    for i in range(G):
        g = ig.unpack(u, vptr, i)
        v0, v1 = int(vptr[i]), int(vptr[i + 1])
        assert np.array_equal(d[v0:v1], orc.bfs(g, 0)), (i, "bfs")
        assert np.array_equal(l[v0:v1], orc.cc(g)), (i, "cc")
        assert int(c[i]) == orc.tc(g), (i, "tc")
        ref, it64, _ = orc.pr_f64(g, iters=int(it[i]))
        assert it64 == int(it[i])
        rel = float(np.abs(s[v0:v1].astype(np.float64) - ref).sum() / ref.sum())
        assert rel <= PR_TOL, (i, "pr", rel)
        worst = max(worst, rel)
    print(f"batched sample: {G} graphs, V {u.nodes}, E {u.edges}; PageRank worst relative L1 {worst:.2e}")


# ------------------------------------------------------------------- served
@pytest.fixture(scope="module")
def served16(ig, gpu):
    g = ig.rmat(16, 16, seed=17, maxw=1000)
    d = ig.DeviceCSR(g)
    srv = ig.Server(d, max_pending=1024)
    yield g, d, srv
    srv.close()
    d.close()


def oracle_answer(ig, orc, g, kind, src, targets):
    dist = orc.bfs(g, int(src)) if kind == 0 else orc.sssp(g, int(src))
    return ig.summarize(kind, src, dist, targets)


def test_served_queries_alone_against_oracle(ig, orc, served16):
    g, d, srv = served16
    rng = np.random.default_rng(3)
    for kind in (0, 1):
        for src in [int(x) for x in g.pick_sources(4, seed=17)] + [int(np.argmin(g.degree()))]:
            tg = rng.integers(0, g.nodes, 8)
            a = srv.wait(srv.submit(kind, src, tg))
            assert a.key() == oracle_answer(ig, orc, g, kind, src, tg).key(), (kind, src)


def test_served_mix_against_oracle(ig, orc, served16):
    """96 BFS and SSSP queries submitted by 4 client threads with staggered
    arrivals share the 64 lanes; every answer equals the oracle's."""
    g, d, srv = served16
    rng = np.random.default_rng(11)
    srcs = g.pick_sources(48, seed=23)
    jobs = [(k, int(s), rng.integers(0, g.nodes, 4)) for k in (0, 1) for s in srcs]
    rng.shuffle(jobs)
    tickets = {}

    def client(part):
        for i in part:
            kind, s, tg = jobs[i]
            tickets[i] = srv.submit(kind, s, tg)
            time.sleep(0.0003 * (i % 4))

    th = [threading.Thread(target=client, args=(range(k, len(jobs), 4),)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i, (kind, s, tg) in enumerate(jobs):
        assert srv.wait(tickets[i]).key() == oracle_answer(ig, orc, g, kind, s, tg).key(), (kind, s)


# -------------------------------------------------------------- edge forms
@pytest.mark.parametrize("name", ["rmat", "road", "er"])
def test_edge_forms_against_oracle(ig, orc, gpu, name):
    g = {"rmat": lambda: ig.rmat(13, 16, seed=7, maxw=1000),
         "road": lambda: ig.road(96, 80, 0.05, 0.001, seed=11, maxw=10000),
         "er": lambda: ig.erdos_renyi(5000, 6.0, seed=13, maxw=255)}[name]()
    sp = g.sp()
    with ig.DeviceCSR(g) as d:
        d_sp = ig.DeviceBuffer.from_array(sp)
        out = np.empty(g.nodes, np.int32)
        for s in (0, g.nodes // 3):
            ig.GPUbfs_edge(s, d, out, sp)
            assert np.array_equal(out, orc.bfs(g, s)), ("bfs", s)
            ig.GPUsssp_edge(s, d, out, sp)
            assert np.array_equal(out, orc.sssp(g, s)), ("sssp", s)
        ig.GPUcc_edge(d, out, sp)
        assert np.array_equal(out, orc.cc(g))
        ig.GPUmis_edge(d, d_sp.ptr, None, out)
        assert np.array_equal(out, orc.mis(g).astype(np.int32))
        count, _ = ig.GPUtc_edge(g.edges, d.nindex_ptr, d.nlist_ptr, d_sp.ptr)
        assert count == orc.tc(g)
        d_sp.close()


# ------------------------------------------------- PageRank, converged FP64
def pr_errors(ig, orc, g, eps):
    s = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
    it, _ = ig.PR_GPU(g, s, g.degree(), eps, 100)
    conv, it_conv, res = orc.pr_f64(g)  # to an L1 residual of 1e-12
    assert res < 1e-12
    same, _, _ = orc.pr_f64(g, iters=it)
    s64 = s.astype(np.float64)
    return it, it_conv, (float(np.abs(s64 - same).sum() / same.sum()),
                         float(np.abs(s64 - conv).sum() / conv.sum()),
                         float(np.abs(s64 - conv).max() / conv.max()))


@pytest.mark.parametrize("name", ["grid256", "rmat16", "road512"])
def test_pagerank_against_converged_fp64(ig, orc, gpu, name):
    g = {"grid256": lambda: ig.grid2d(256, 256, maxw=255, seed=1),
         "rmat16": lambda: ig.rmat(16, 16, seed=7, maxw=1000),
         "road512": lambda: ig.road(512, 512, 0.05, 0.001, seed=11, maxw=10000)}[name]()
    it6, itc, (same6, conv6, max6) = pr_errors(ig, orc, g, 1e-6)
    it7, _, (same7, conv7, max7) = pr_errors(ig, orc, g, 1e-7)
    print(f"{name}: eps 1e-6: {it6} it, rel L1 vs same-iteration FP64 {same6:.2e}, vs converged ({itc} it) "
          f"{conv6:.2e}, max {max6:.2e}; eps 1e-7: {it7} it, vs converged {conv7:.2e}, max {max7:.2e}")
    assert same6 <= PR_TOL and same7 <= PR_TOL  # arithmetic error
    assert conv7 <= PR_TOL  # total error once run to a residual of 1e-7
    assert conv6 <= 1e-5  # truncation error of the 1e-6 stopping rule: a few 1e-6
