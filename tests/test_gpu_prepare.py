"""Device-side graph preparation (ig_csr_prepare): a graph with shuffled
adjacency lists, missing reverse edges, duplicate edges (heavier copies) and
self loops comes back exactly as the clean symmetric graph it was made from;
the (degree, id) relabelling equals the host ig_degree_order bit for bit, and
triangle counting on the prepared graph gives the same count."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def messy(ig, g, seed):
    """g with every list shuffled, one direction of ~10% of the undirected
    edges removed, ~5% of the edges duplicated with a larger weight and self
    loops on ~1% of the vertices."""
    rng = np.random.default_rng(seed)
    src = np.repeat(np.arange(g.nodes, dtype=np.int64), g.degree())
    dst = g.nlist.astype(np.int64)
    w = g.eweight.astype(np.int64) if g.eweight is not None else np.zeros(g.edges, np.int64)
    drop = (src < dst) & (rng.random(g.edges) < 0.1)
    keep = ~drop
    src, dst, w = src[keep], dst[keep], w[keep]
    dup = rng.random(src.size) < 0.05
    loops = rng.choice(g.nodes, max(1, g.nodes // 100), replace=False)
    src = np.concatenate([src, src[dup], loops])
    dst = np.concatenate([dst, dst[dup], loops])
    w = np.concatenate([w, w[dup] + 5, np.full(loops.size, 7)])
    order = np.lexsort((rng.random(src.size), src))  # grouped by source, shuffled within
    src, dst, w = src[order], dst[order], w[order]
    nindex = np.concatenate([[0], np.cumsum(np.bincount(src, minlength=g.nodes))]).astype(np.int32)
    ew = w.astype(np.int32) if g.eweight is not None else None
    return ig.Graph(nindex, dst.astype(np.int32), ew)


def same(a, b):
    assert a.nodes == b.nodes and a.edges == b.edges
    assert np.array_equal(a.nindex, b.nindex)
    assert np.array_equal(a.nlist, b.nlist)
    if a.eweight is None or b.eweight is None:
        assert a.eweight is None and b.eweight is None
    else:
        assert np.array_equal(a.eweight, b.eweight)


@pytest.mark.parametrize("name", ["rmat12", "road64", "grid", "er4k_unweighted"])
def test_prepare_restores_clean_graph(ig, gpu, name):
    g = {"rmat12": lambda: ig.rmat(12, 16, seed=7, maxw=1000),
         "road64": lambda: ig.road(64, 64, 0.05, 0.001, seed=11, maxw=10000),
         "grid": lambda: ig.grid2d(40, 30, maxw=255),
         "er4k_unweighted": lambda: ig.erdos_renyi(4096, 8.0, seed=3)}[name]()
    m = messy(ig, g, seed=5)
    assert m.edges != g.edges
    with ig.DeviceCSR(m) as d:
        p = d.prepare(symmetrize=True)
        try:
            same(p.to_graph(), g)
        finally:
            p.close()
        with ig.DeviceCSR(g) as dg:
            q = dg.prepare(degree_order=True)
            try:
                same(q.to_graph(), g.degree_ordered())
            finally:
                q.close()


def test_prepare_in_one_pass_and_tc(ig, gpu):
    """Symmetrise + clean + degree order in one call equals the host order of
    the clean graph, and TC on it matches TC on the host-prepared graph."""
    g = ig.rmat(14, 16, seed=7, maxw=1000)
    host = g.degree_ordered()
    with ig.DeviceCSR(messy(ig, g, seed=9)) as d:
        p = d.prepare(symmetrize=True, degree_order=True)
        try:
            same(p.to_graph(), host)
            count, _ = ig.GPUtc_vertex(p.nodes, p.nindex_ptr, p.nlist_ptr)
        finally:
            p.close()
    with ig.DeviceCSR(host) as dh:
        ref, _ = ig.GPUtc_vertex(dh.nodes, dh.nindex_ptr, dh.nlist_ptr)
    assert count == ref


def test_prepare_rmat20_degree_order(ig, gpu):
    g = ig.rmat(20, 16, seed=7, maxw=1000)
    with ig.DeviceCSR(g) as d:
        q = d.prepare(degree_order=True)
        try:
            same(q.to_graph(), g.degree_ordered())
        finally:
            q.close()


def test_prepare_edgeless_and_bad_flags(ig, gpu):
    g = ig.Graph(np.zeros(6, np.int32), np.zeros(0, np.int32), None)
    with ig.DeviceCSR(g) as d:
        p = d.prepare(symmetrize=True, degree_order=True)
        try:
            h = p.to_graph()
            assert h.nodes == 5 and h.edges == 0 and np.array_equal(h.nindex, np.zeros(6, np.int32))
        finally:
            p.close()
        out = ig.CSR()
        import ctypes
        assert ig.load().ig_csr_prepare(ctypes.byref(d.c), 8, ctypes.byref(out)) != 0
