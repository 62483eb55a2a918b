"""The oracle's copy of the benchmark workload generator (oracle/workload.c),
which the CPU arms of the benchmark use so that they load no GPU library,
produces exactly the library's graphs: the same CSR arrays and weights, the
same (degree, id) relabelling and the same sources."""
import numpy as np
import pytest


@pytest.mark.parametrize("scale,ef,permute,maxw", [(10, 16, True, 1000), (13, 16, True, 1000), (12, 8, False, 255),
                                                    (14, 16, True, 0)])
def test_rmat_generator_identical(ig, orc, scale, ef, permute, maxw):
    a = ig.rmat(scale, ef, 0.57, 0.19, 0.19, seed=7, maxw=maxw, permute=permute)
    b = orc.gen_rmat(scale, ef, 0.57, 0.19, 0.19, seed=7, maxw=maxw, permute=permute, threads=3)
    assert np.array_equal(a.nindex, b.nindex)
    assert np.array_equal(a.nlist, b.nlist)
    if maxw:
        assert np.array_equal(a.eweight, b.eweight)
    else:
        assert b.eweight is None
    assert np.array_equal(a.pick_sources(16, seed=7), b.pick_sources(16, seed=7))


def test_degree_order_identical(ig, orc):
    a = ig.rmat(13, 16, seed=7, maxw=1000, permute=True)
    b = orc.gen_rmat(13, 16, seed=7, maxw=1000, permute=True, threads=4)
    da, db = a.degree_ordered(), b.degree_ordered(threads=2)
    assert np.array_equal(da.nindex, db.nindex)
    assert np.array_equal(da.nlist, db.nlist)
    assert np.array_equal(da.eweight, db.eweight)


def test_egr_writer_matches_library(ig, orc, tmp_path):
    b = orc.gen_rmat(9, 16, seed=3, maxw=50, threads=2)
    p = tmp_path / "g.egr"
    b.write_egr(str(p))
    g = ig.read_egr(str(p))
    assert np.array_equal(g.nindex, b.nindex) and np.array_equal(g.nlist, b.nlist)
    assert np.array_equal(g.eweight, b.eweight)
