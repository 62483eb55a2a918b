"""Batch packing and the batch generator (host only)."""
import numpy as np

from conftest import kat_graphs


def test_pack_unpack_roundtrip(ig):
    K = kat_graphs(ig)
    gs = [K["single"], K["path"], K["two_isolated"], K["complete"], ig.grid2d(5, 7, maxw=9)]
    for g in gs:
        if g.eweight is None:
            g.eweight = np.ones(g.edges, np.int32)
    u, vptr = ig.pack(gs)
    assert u.nodes == sum(g.nodes for g in gs) and u.edges == sum(g.edges for g in gs)
    for i, g in enumerate(gs):
        h = ig.unpack(u, vptr, i)
        assert np.array_equal(h.nindex, g.nindex) and np.array_equal(h.nlist, g.nlist)
        assert np.array_equal(h.eweight, g.eweight)


def test_gen_batch_structure(ig):
    u, vptr = ig.gen_batch(24, vmin=64, vmax=4096, seed=13)
    assert len(vptr) == 25 and vptr[0] == 0 and vptr[-1] == u.nodes
    sizes = np.diff(vptr)
    assert sizes.min() >= 64 and sizes.max() <= 4096
    for i in range(24):
        g = ig.unpack(u, vptr, i)
        assert g.is_sorted()
        src = np.repeat(np.arange(g.nodes), g.degree())
        assert not np.any(src == g.nlist)
        assert np.all((g.nlist >= 0) & (g.nlist < g.nodes))  # no edge leaves its graph
    u2, vptr2 = ig.gen_batch(24, vmin=64, vmax=4096, seed=13)
    assert u.digest() == u2.digest() and np.array_equal(vptr, vptr2)
