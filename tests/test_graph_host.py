"""Host-side graph layer: generators, .egr I/O (format of include/ECLgraph.h)
and its error behaviour, degree ordering, sources.  No GPU."""
import ctypes
import os

import numpy as np
import pytest


def _symmetric(g):
    src = np.repeat(np.arange(g.nodes), g.degree())
    fwd = set(zip(src.tolist(), g.nlist.tolist()))
    return all((v, u) in fwd for (u, v) in fwd)


def test_grid256_matches_config_size(ig):
    g = ig.grid2d(256, 256, maxw=255, seed=1)
    assert (g.nodes, g.edges) == (65536, 261120)
    assert g.is_sorted()
    assert g.eweight.min() >= 1 and g.eweight.max() <= 255


def test_grid_adjacency_and_weights_symmetric(ig):
    g = ig.grid2d(9, 7, maxw=100, seed=5)
    assert _symmetric(g)
    w = {}
    src = np.repeat(np.arange(g.nodes), g.degree())
    for u, v, x in zip(src, g.nlist, g.eweight):
        w[(u, v)] = x
    assert all(w[(v, u)] == x for (u, v), x in w.items())


@pytest.mark.parametrize("maker", ["rmat", "road", "er"])
def test_generators_simple_symmetric_sorted(ig, maker):
    g = {"rmat": lambda: ig.rmat(10, 8, seed=3, maxw=1000),
         "road": lambda: ig.road(30, 20, 0.05, 0.01, seed=11, maxw=10000),
         "er": lambda: ig.erdos_renyi(2000, 8.0, seed=13, maxw=255)}[maker]()
    assert g.is_sorted()
    src = np.repeat(np.arange(g.nodes), g.degree())
    assert not np.any(src == g.nlist)  # no self loops
    assert _symmetric(g)
    assert g.eweight.min() >= 1


def test_generators_deterministic(ig):
    assert ig.rmat(11, 16, seed=7).digest() == ig.rmat(11, 16, seed=7).digest()
    assert ig.rmat(11, 16, seed=7).digest() != ig.rmat(11, 16, seed=8).digest()


def test_golden_graph_digests(ig, golden):
    from conftest import golden_graphs
    meta, _ = golden
    makers = golden_graphs(ig)
    for name, m in list(meta["graphs"].items()) + list(meta["digest_only"].items()):
        assert str(makers[name]().digest()) == m["digest"], name


def test_road_deletes_and_adds(ig):
    full = ig.grid2d(100, 100)
    r = ig.road(100, 100, 0.05, 0.001, seed=11, maxw=10000)
    assert 0.9 * full.edges < r.edges < full.edges


def test_egr_roundtrip(ig, tmp_path):
    g = ig.rmat(9, 8, seed=2, maxw=50)
    p = tmp_path / "g.egr"
    g.write_egr(str(p))
    h = ig.read_egr(str(p))
    assert np.array_equal(g.nindex, h.nindex) and np.array_equal(g.nlist, h.nlist)
    assert np.array_equal(g.eweight, h.eweight)
    # unweighted: the reader returns eweight = NULL (include/ECLgraph.h:70-76)
    u = ig.grid2d(5, 5)
    u.write_egr(str(p))
    assert ig.read_egr(str(p)).eweight is None
    # byte layout: int nodes, int edges, nindex, nlist
    raw = np.fromfile(str(p), dtype=np.int32)
    assert raw[0] == 25 and raw[1] == u.edges and np.array_equal(raw[2:2 + 26], u.nindex)


def test_egr_errors(ig, tmp_path):
    with pytest.raises(ig.IndigoError) as e:
        ig.read_egr(str(tmp_path / "missing.egr"))
    assert e.value.status == ig._lib.IG_ERR_IO
    p = tmp_path / "bad.egr"
    np.array([0, 5], np.int32).tofile(str(p))  # node count too low
    with pytest.raises(ig.IndigoError) as e:
        ig.read_egr(str(p))
    assert e.value.status == ig._lib.IG_ERR_FORMAT
    g = ig.grid2d(4, 4)
    g.write_egr(str(p))
    data = p.read_bytes()
    p.write_bytes(data[: len(data) // 2])  # truncated
    with pytest.raises(ig.IndigoError):
        ig.read_egr(str(p))
    np.concatenate([np.array([3, 2], np.int32), np.array([0, 1, 2, 2], np.int32),
                    np.array([1, 7], np.int32)]).tofile(str(p))  # neighbour out of range
    with pytest.raises(ig.IndigoError) as e:
        ig.read_egr(str(p))
    assert e.value.status == ig._lib.IG_ERR_FORMAT


def test_degree_order(ig, orc):
    g = ig.rmat(10, 16, seed=7, maxw=9)
    d = g.degree_ordered()
    assert d.is_sorted() and d.edges == g.edges
    assert np.all(np.diff(d.degree()) >= 0)
    assert orc.tc(d) == orc.tc(g)


def test_pick_sources(ig):
    g = ig.rmat(12, 16, seed=7)
    s = g.pick_sources(16, seed=7)
    assert len(set(s.tolist())) == 16 and np.all(g.degree()[s] > 0)
    assert np.array_equal(s, g.pick_sources(16, seed=7))


def test_sp_array(ig):
    g = ig.grid2d(3, 3)
    sp = g.sp()
    assert sp.shape[0] == g.edges and np.all(np.diff(sp) >= 0) and sp[-1] == g.nodes - 1


def test_check_sorted_detects(ig):
    g = ig.grid2d(4, 4)
    nl = g.nlist.copy()
    nl[0], nl[1] = nl[1], nl[0]
    assert not ig.Graph(g.nindex, nl).is_sorted()
