"""The allocation-free BFS entry point (ig_bfs_vertex_noalloc), for callers
that cannot call cudaMalloc: its scratch is a fixed array in the library's
device image.  Checked through the C ABI against the allocating entry point
ig_bfs_vertex and against the oracle (BFS levels are integers: the
comparisons are exact), on two calls in a row, so that a call that finds the
previous call's data in the shared array still gives the right answer; and
the device's free memory is the same before and after calls that follow the
first one on the device.  This file is collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_NODES = 1 << 20


def _noalloc(ig, src, d, out):
    ig.check(ig.load().ig_bfs_vertex_noalloc(src, ctypes.byref(d.c), out.ptr, None))
    return out.to_array(np.int32, d.nodes)


def test_noalloc_matches_dropin_and_oracle_twice(ig, orc, gpu):
    g = ig.rmat(16, 16, seed=7)  # 65,536 vertices, hubs above the grid-wide threshold
    srcs = [int(s) for s in g.pick_sources(2, seed=3)]
    with ig.DeviceCSR(g) as d:
        out = ig.DeviceBuffer(4 * g.nodes)
        for s in srcs:  # two calls in a row, different sources
            ref = np.empty(g.nodes, np.int32)
            ig.GPUbfs_vertex(s, d, ref)
            got = _noalloc(ig, s, d, out)
            assert np.array_equal(got, ref)
            assert np.array_equal(got, orc.bfs(g, s))
        # and the first source again, after the array holds the second run's data
        ref = np.empty(g.nodes, np.int32)
        ig.GPUbfs_vertex(srcs[0], d, ref)
        assert np.array_equal(_noalloc(ig, srcs[0], d, out), ref)


def test_noalloc_high_diameter_graph(ig, orc, gpu):
    g = ig.grid2d(512, 256)  # 131,072 vertices, 766 levels
    with ig.DeviceCSR(g) as d:
        out = ig.DeviceBuffer(4 * g.nodes)
        ref = np.empty(g.nodes, np.int32)
        ig.GPUbfs_vertex(0, d, ref)
        for _ in range(2):
            got = _noalloc(ig, 0, d, out)
            assert np.array_equal(got, ref)
        assert np.array_equal(got, orc.bfs(g, 0))


def test_noalloc_leaves_free_memory_unchanged(ig, gpu):
    """Any device allocation would lower the free memory by at least one
    allocation granule; the calls after the first one on the device (which
    looks up the array's address) change nothing."""
    L = ig.load()

    def free_bytes():
        f, t = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        ig.check(L.ig_device_memory(ctypes.byref(f), ctypes.byref(t)))
        assert 0 < f.value <= t.value
        return f.value

    g = ig.rmat(15, 16, seed=5)
    with ig.DeviceCSR(g) as d:
        out = ig.DeviceBuffer(4 * g.nodes)
        _noalloc(ig, 0, d, out)
        free0 = free_bytes()
        for s in (1, 2, 3):
            _noalloc(ig, s, d, out)
        free1 = free_bytes()
    assert free1 == free0


def test_noalloc_rejects_graphs_over_the_limit(ig, gpu):
    # checked before any device access: the pointers are never dereferenced
    c = ig.CSR()
    c.nodes, c.edges = MAX_NODES + 1, 0
    dummy = (ctypes.c_int * 1)()
    c.nindex = ctypes.cast(dummy, ctypes.POINTER(ctypes.c_int))
    c.nlist = ctypes.cast(dummy, ctypes.POINTER(ctypes.c_int))
    st = ig.load().ig_bfs_vertex_noalloc(0, ctypes.byref(c), ctypes.cast(dummy, ctypes.c_void_p), None)
    assert st == ig._lib.IG_ERR_INVALID_ARG
    assert b"exceed" in ig.load().ig_last_error()
