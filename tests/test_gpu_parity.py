"""GPU parity: every drop-in entry point (through the C ABI) against the
oracle and the reference's golden fixtures -- bit-exact for BFS/SSSP/CC/MIS/TC,
FP32 PageRank within 1e-6 relative L1 of the FP64 oracle run for the same
number of iterations."""
import ctypes
import hashlib
import math

import numpy as np
import pytest

from conftest import golden_graphs, kat_graphs

pytestmark = pytest.mark.gpu

INT_MAX = 2147483647
PR_TOL = 1e-6  # relative L1 against FP64, same iteration count


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def graphs(ig, gpu):
    out = {k: v() for k, v in golden_graphs(ig).items()}
    out.update(kat_graphs(ig))
    out["rmat14"] = ig.rmat(14, 16, seed=7, maxw=1000)
    out["road128"] = ig.road(128, 96, 0.05, 0.001, seed=11, maxw=10000)
    out["rmat18"] = ig.rmat(18, 16, seed=7, maxw=1000)
    return out


def run_all(ig, g, sources):
    """Runs the six drop-ins on g; returns a dict of host results."""
    res = {}
    with ig.DeviceCSR(g) as d:
        for k, s in enumerate(sources):
            dist = np.empty(g.nodes, np.int32)
            ig.GPUbfs_vertex(int(s), d, dist)
            res[f"bfs{k}"] = dist
            if g.eweight is not None:
                dist = np.empty(g.nodes, np.int32)
                ig.GPUsssp_vertex(int(s), d, dist)
                res[f"sssp{k}"] = dist
        lab = np.empty(g.nodes, np.int32)
        ig.GPUcc_vertex(d, lab)
        res["cc"] = lab
        st = np.empty(g.nodes, np.int32)
        ig.GPUmis_vertex(d, None, st)
        res["mis"] = st
        if g.is_sorted():
            res["tc"] = ig.GPUtc_vertex(g.nodes, d.nindex_ptr, d.nlist_ptr)[0]
    return res


@pytest.mark.parametrize("name", ["grid64", "rmat12", "road64", "er4k", "rmat12_dord"])
def test_dropins_match_reference_fixtures(ig, golden, graphs, name):
    _, A = golden
    g = graphs[name]
    srcs = A[f"{name}/sources"]
    r = run_all(ig, g, srcs)
    for k in range(len(srcs)):
        assert np.array_equal(r[f"bfs{k}"], A[f"{name}/bfs{k}"]), f"bfs{k}"
        assert np.array_equal(r[f"sssp{k}"], A[f"{name}/sssp{k}"]), f"sssp{k}"
    assert np.array_equal(r["cc"], A[f"{name}/cc"])
    assert np.array_equal(r["mis"], A[f"{name}/mis"].astype(np.int32))
    assert r["tc"] == int(A[f"{name}/tc"][0])


def test_grid256_config_digests(ig, golden, graphs):
    meta, _ = golden
    m = meta["digest_only"]["grid256"]
    g = graphs["grid256"]
    r = run_all(ig, g, m["sources"])
    for k in range(len(m["sources"])):
        assert sha(r[f"bfs{k}"]) == m["sha256"][f"bfs{k}"]
        assert sha(r[f"sssp{k}"]) == m["sha256"][f"sssp{k}"]
    assert sha(r["cc"]) == m["sha256"]["cc"]
    assert sha(r["mis"].astype(np.uint8)) == m["sha256"]["mis"]
    assert r["tc"] == 0


@pytest.mark.parametrize("name", ["single", "two_isolated", "edge", "path", "star", "complete", "two_grids",
                                  "hubby", "rmat14", "road128"])
def test_dropins_match_oracle(ig, orc, graphs, name):
    g = graphs[name]
    srcs = [0, g.nodes - 1, g.nodes // 2] if g.nodes > 2 else list(range(g.nodes))
    r = run_all(ig, g, srcs)
    for k, s in enumerate(srcs):
        assert np.array_equal(r[f"bfs{k}"], orc.bfs(g, int(s))), f"bfs src {s}"
        if g.eweight is not None:
            assert np.array_equal(r[f"sssp{k}"], orc.sssp(g, int(s))), f"sssp src {s}"
    assert np.array_equal(r["cc"], orc.cc(g))
    assert np.array_equal(r["mis"], orc.mis(g).astype(np.int32))
    assert r["tc"] == orc.tc(g)


def test_known_answers_on_gpu(ig, graphs):
    g = ig.grid2d(300, 200)
    r = run_all(ig, g, [0])
    y, x = np.divmod(np.arange(g.nodes), 300)
    assert np.array_equal(r["bfs0"], x + y)
    assert r["tc"] == 0 and np.all(r["cc"] == 0)
    k = graphs["complete"]
    assert run_all(ig, k, [0])["tc"] == math.comb(k.nodes, 3)


def test_unreachable_is_int_max(ig, graphs):
    g = graphs["two_grids"]
    r = run_all(ig, g, [0])
    assert np.all(r["bfs0"][100:] == INT_MAX) and np.all(r["sssp0"][100:] == INT_MAX)
    assert np.all(r["bfs0"][:100] < INT_MAX)


@pytest.mark.parametrize("name", ["grid64", "rmat12", "er4k", "rmat14", "hubby", "star"])
def test_pagerank_fp32_against_fp64(ig, orc, graphs, name):
    g = graphs[name]
    deg = g.degree()
    scores = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
    it, _ = ig.PR_GPU(g, scores, deg, epsilon=1e-6, max_iter=100)
    ref, it64, _ = orc.pr_f64(g, iters=it)
    assert it64 == it
    rel_l1 = np.abs(scores.astype(np.float64) - ref).sum() / np.abs(ref).sum()
    assert rel_l1 <= PR_TOL, rel_l1
    # iteration count agrees with the reference FP32 algorithm to within one,
    # unless the uncompensated FP32 sum never gets below epsilon (it then
    # stops at max_iter, e.g. on the bipartite star, while Kahan converges)
    _, it32, _ = orc.pr_f32(g, 1e-6, 100)
    assert abs(it32 - it) <= 1 or (it32 == 100 and it < 100)


def test_pagerank_reference_constants(ig, orc, golden, graphs):
    """EPSILON 1e-4 / MAX_ITER 100 as in include/pr_cuda.h: same iteration
    count as the reference program and scores within tolerance of it."""
    _, A = golden
    g = graphs["rmat12"]
    scores = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
    it, _ = ig.PR_GPU(g, scores, g.degree())
    _, it_ref, _ = orc.pr_f32(g, 1e-4, 100)
    assert abs(it - it_ref) <= 1
    ref = A["rmat12/pr"].astype(np.float64)
    assert np.abs(scores - ref).sum() / ref.sum() < 1e-5


def test_pagerank_deterministic(ig, graphs):
    g = graphs["rmat14"]
    outs = []
    for _ in range(2):
        s = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
        ig.PR_GPU(g, s, g.degree(), 1e-6, 100)
        outs.append(s)
    assert np.array_equal(outs[0], outs[1])


def test_pagerank_hub_split_path(ig, orc, graphs):
    """Forces the chunked hub path (hub degree 64, chunks of 32 edges)."""
    g = graphs["rmat14"]
    old = (ig.get_option("pr_hub_degree"), ig.get_option("pr_chunk"))
    try:
        ig.set_option("pr_hub_degree", 64)
        ig.set_option("pr_chunk", 32)
        s = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
        it, _ = ig.PR_GPU(g, s, g.degree(), 1e-6, 100)
    finally:
        ig.set_option("pr_hub_degree", old[0])
        ig.set_option("pr_chunk", old[1])
    ref, _, _ = orc.pr_f64(g, iters=it)
    assert np.abs(s - ref).sum() / ref.sum() <= PR_TOL


def test_hub_paths_forced(ig, orc, graphs):
    """Small hub degree sends many vertices through the grid-wide hub
    expansion of BFS / SSSP / CC."""
    g = graphs["rmat14"]
    old = ig.get_option("hub_degree")
    try:
        ig.set_option("hub_degree", 32)
        r = run_all(ig, g, [0, 5])
    finally:
        ig.set_option("hub_degree", old)
    for k, s in enumerate([0, 5]):
        assert np.array_equal(r[f"bfs{k}"], orc.bfs(g, s))
        assert np.array_equal(r[f"sssp{k}"], orc.sssp(g, s))
    assert np.array_equal(r["cc"], orc.cc(g))


@pytest.mark.parametrize("alpha,beta", [(1, 1), (1000000, 24), (2, 1000000)])
def test_bfs_direction_settings(ig, orc, graphs, alpha, beta):
    g = graphs["rmat14"]
    old = (ig.get_option("bfs_alpha"), ig.get_option("bfs_beta"))
    try:
        ig.set_option("bfs_alpha", alpha)
        ig.set_option("bfs_beta", beta)
        r = run_all(ig, g, [3])
    finally:
        ig.set_option("bfs_alpha", old[0])
        ig.set_option("bfs_beta", old[1])
    assert np.array_equal(r["bfs0"], orc.bfs(g, 3))


def test_degree_ordered_ids_match_oracle(ig, orc, graphs):
    """Ids in (degree, id) order: consecutive runs of high-degree vertices
    (MIS chunk scheduling), the TC orientation without degree lookups and the
    exact-bitmap count, SSSP and BFS on the same relabelled graph."""
    g = graphs["rmat14"].degree_ordered()
    srcs = [0, g.nodes - 1, g.nodes // 2]
    r = run_all(ig, g, srcs)
    for k, s in enumerate(srcs):
        assert np.array_equal(r[f"bfs{k}"], orc.bfs(g, int(s))), f"bfs src {s}"
        assert np.array_equal(r[f"sssp{k}"], orc.sssp(g, int(s))), f"sssp src {s}"
    assert np.array_equal(r["cc"], orc.cc(g))
    assert np.array_equal(r["mis"], orc.mis(g).astype(np.int32))
    assert r["tc"] == orc.tc(g)


@pytest.mark.parametrize("scale,degree", [(0, 16), (1, 16), (64, 0), (8, 1000000)])
def test_sssp_window_settings(ig, orc, graphs, scale, degree):
    """The degree window (a queued vertex of degree d is expanded once its
    distance is below the round minimum + C/d) only reorders work: off, very
    narrow, applied to every vertex, or to none, the distances are exact."""
    old = (ig.get_option("sssp_window_scale"), ig.get_option("sssp_window_degree"))
    try:
        ig.set_option("sssp_window_scale", scale)
        ig.set_option("sssp_window_degree", degree)
        for name in ("rmat14", "hubby", "road128"):
            g = graphs[name]
            srcs = [0, g.nodes // 2]
            with ig.DeviceCSR(g) as d:
                for s in srcs:
                    dist = np.empty(g.nodes, np.int32)
                    ig.GPUsssp_vertex(int(s), d, dist)
                    assert np.array_equal(dist, orc.sssp(g, int(s))), f"{name} src {s}"
    finally:
        ig.set_option("sssp_window_scale", old[0])
        ig.set_option("sssp_window_degree", old[1])


@pytest.mark.parametrize("delta", [1, 7, 1000, 100000000])
def test_sssp_bucket_widths(ig, orc, graphs, delta):
    g = graphs["road128"]
    old = ig.get_option("sssp_delta")
    try:
        ig.set_option("sssp_delta", delta)
        r = run_all(ig, g, [0])
    finally:
        ig.set_option("sssp_delta", old)
    assert np.array_equal(r["sssp0"], orc.sssp(g, 0))


def test_edge_forms_equal_vertex_forms(ig, graphs):
    g = graphs["rmat12"]
    sp = g.sp()
    with ig.DeviceCSR(g) as d:
        a = np.empty(g.nodes, np.int32)
        b = np.empty(g.nodes, np.int32)
        ig.GPUbfs_vertex(5, d, a)
        ig.GPUbfs_edge(5, d, b, sp)
        assert np.array_equal(a, b)
        ig.GPUsssp_vertex(5, d, a)
        ig.GPUsssp_edge(5, d, b, sp)
        assert np.array_equal(a, b)
        ig.GPUcc_vertex(d, a)
        ig.GPUcc_edge(d, b, sp)
        assert np.array_equal(a, b)


def test_device_api_matches_dropins(ig, graphs):
    g = graphs["rmat14"]
    r = run_all(ig, g, [7])
    with ig.DeviceCSR(g) as d:
        dg = ig.DeviceGraph(d)
        buf = ig.DeviceBuffer(4 * g.nodes)
        dg.bfs(7, buf)
        assert dg.last_run().status == 0
        assert np.array_equal(buf.to_array(np.int32, g.nodes), r["bfs0"])
        dg.sssp(7, buf)
        assert np.array_equal(buf.to_array(np.int32, g.nodes), r["sssp0"])
        dg.cc(buf)
        assert np.array_equal(buf.to_array(np.int32, g.nodes), r["cc"])
        dg.mis(buf)
        assert np.array_equal(buf.to_array(np.int32, g.nodes), r["mis"])
        cnt = ig.DeviceBuffer(8)
        dg.tc(cnt)
        assert int(cnt.to_array(np.uint64, 1)[0]) == r["tc"]
        sc = ig.DeviceBuffer.from_array(np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32))
        dg.pagerank(sc, 1e-6, 100)
        info = dg.last_run()
        assert info.status == 0 and info.iterations > 1 and info.residual < 1e-6
        dg.close()


def test_tc_rejects_unsorted(ig, graphs):
    g = graphs["grid64"]
    nl = g.nlist.copy()
    nl[0], nl[1] = nl[1], nl[0]
    bad = ig.Graph(g.nindex, nl)
    with ig.DeviceCSR(bad) as d:
        with pytest.raises(ig.IndigoError) as e:
            ig.GPUtc_vertex(bad.nodes, d.nindex_ptr, d.nlist_ptr)
        assert e.value.status == ig._lib.IG_ERR_UNSORTED
        # the context stays usable after the error
        dist = np.empty(bad.nodes, np.int32)
        ig.GPUbfs_vertex(0, d, dist)
        assert dist[0] == 0


@pytest.mark.parametrize("where", ["hub", "light"])
def test_tc_rejects_unsorted_ranked(ig, orc, graphs, where):
    """Ids in (degree, id) order: a swapped pair in a hub's list (checked by
    the chunked hub copy) or in a short list (checked by the count pass) is
    reported as unsorted; the sorted input counts right."""
    g = graphs["rmat18"].degree_ordered()
    deg = np.diff(g.nindex)
    with ig.DeviceCSR(g) as d:
        assert ig.GPUtc_vertex(g.nodes, d.nindex_ptr, d.nlist_ptr)[0] == orc.tc(g)
    v = int(np.argmax(deg)) if where == "hub" else int(np.argmax((deg > 2) & (deg < 64)))
    assert (deg[v] > 256) == (where == "hub")
    nl = g.nlist.copy()
    b = int(g.nindex[v]) + int(deg[v]) // 2
    nl[b], nl[b + 1] = nl[b + 1], nl[b]
    bad = ig.Graph(g.nindex, nl)
    with ig.DeviceCSR(bad) as d:
        with pytest.raises(ig.IndigoError) as e:
            ig.GPUtc_vertex(bad.nodes, d.nindex_ptr, d.nlist_ptr)
        assert e.value.status == ig._lib.IG_ERR_UNSORTED


def test_bounded_wait_reports_timeout(ig, graphs):
    """A grid barrier that one block never reaches ends in IG_ERR_TIMEOUT
    after the bound, and the device keeps working afterwards."""
    L = ig.load()
    st = ctypes.c_int(-1)
    ig.check(L.ig_selftest_wait_timeout(200, ctypes.byref(st)))
    assert st.value == ig._lib.IG_ERR_TIMEOUT
    g = graphs["grid64"]
    with ig.DeviceCSR(g) as d:
        dist = np.empty(g.nodes, np.int32)
        ig.GPUbfs_vertex(0, d, dist)
        assert dist.max() == 126


def test_repeated_calls_reuse_scratch(ig, orc, graphs):
    """Alternating graph sizes exercise the grow-only scratch pool."""
    for name in ["rmat14", "grid64", "rmat14", "path"]:
        g = graphs[name]
        with ig.DeviceCSR(g) as d:
            dist = np.empty(g.nodes, np.int32)
            ig.GPUbfs_vertex(0, d, dist)
            assert np.array_equal(dist, orc.bfs(g, 0))


def test_random_gather_probe(ig, gpu):
    """The calibration kernel runs and gives a finite positive rate; it
    rejects tables beyond its 32-bit index range."""
    rate = ig.probe_random_gather(1 << 20, 1 << 22, 1)
    assert math.isfinite(rate) and rate > 0
    with pytest.raises(ig.IndigoError):
        ig.probe_random_gather(1 << 33, 1 << 20, 1)


@pytest.mark.parametrize("merge_below,spin", [(2147483647, 0), (2147483647, 1000), (65536, 1000), (0, 1000)])
def test_sssp_item_pass_forms(ig, orc, graphs, merge_below, spin):
    """Work items expanded in the round that makes them (one grid barrier per
    round) in every round, in rounds below the default frontier size, or
    after a second barrier in every round: the distances are exact each
    way.  Degree 4 as the item threshold makes almost every list work items;
    on RMAT-18 with 32-edge items a merged round holds more than the 65,536
    items of its small list, so the rest go through the second barrier."""
    old = {k: ig.get_option(k) for k in ("sssp_merge_below", "sssp_spin_ns", "sssp_warp_degree", "sssp_item_edges")}
    try:
        ig.set_option("sssp_merge_below", merge_below)
        ig.set_option("sssp_spin_ns", spin)
        cases = [(64, 256, n) for n in ("rmat14", "hubby", "road128", "star")] + \
                [(4, 256, n) for n in ("rmat14", "hubby", "road128", "star")] + [(1, 32, "rmat18")]
        for wd, ie, name in cases:
            ig.set_option("sssp_warp_degree", wd)
            ig.set_option("sssp_item_edges", ie)
            g = graphs[name]
            with ig.DeviceCSR(g) as d:
                for s in (0, g.nodes // 2):
                    dist = np.empty(g.nodes, np.int32)
                    ig.GPUsssp_vertex(int(s), d, dist)
                    assert np.array_equal(dist, orc.sssp(g, int(s))), f"{name} src {s} wd {wd}"
    finally:
        for k, v in old.items():
            ig.set_option(k, v)


@pytest.mark.parametrize("opt,values", [("bfs_bitmap", (0, 1)), ("cc_rounds", (0, 1, 2)), ("cc_bfs_seed", (0, 1))])
def test_traversal_option_forms_match_oracle(ig, orc, graphs, opt, values):
    """BFS with and without the level bitmaps of its bottom-up levels (pulling
    from the first level too), CC with the sampled neighbours linked in one
    pass, one round each or after flattening, and CC whose largest-degree
    component is labelled by a BFS: the results are exact every way."""
    old = {k: ig.get_option(k) for k in (opt, "bfs_alpha")}
    try:
        for val in values:
            ig.set_option(opt, val)
            for alpha in (14, 1):
                ig.set_option("bfs_alpha", alpha)
                for name in ("rmat14", "hubby", "road128", "two_grids", "star", "single", "two_isolated", "er4k"):
                    g = graphs[name]
                    r = run_all(ig, g, [0, g.nodes // 2])
                    for k, s in enumerate([0, g.nodes // 2]):
                        assert np.array_equal(r[f"bfs{k}"], orc.bfs(g, s)), (opt, val, alpha, name, s)
                    assert np.array_equal(r["cc"], orc.cc(g)), (opt, val, name)
    finally:
        for k, v in old.items():
            ig.set_option(k, v)


@pytest.mark.parametrize("subwarp,prefetch,two", [(1, 1, 1), (0, 0, 0), (1, 0, 0), (0, 1, 1)])
def test_pagerank_gather_forms(ig, orc, graphs, subwarp, prefetch, two):
    """Medium lists summed by 8-lane sub-warps or by the whole warp, with or
    without the L2 prefetch, contributions gathered in a dense first pass or
    while summing: within 1e-6 relative L1 of FP64, deterministic, and the
    two-pass form gives the same bits as the one-pass form."""
    old = (ig.get_option("pr_subwarp"), ig.get_option("pr_prefetch"), ig.get_option("pr_two_pass"))
    try:
        ig.set_option("pr_subwarp", subwarp)
        ig.set_option("pr_prefetch", prefetch)
        ig.set_option("pr_two_pass", 1 - two)
        other = {}
        for name in ("rmat14", "hubby"):
            g = graphs[name]
            s = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
            ig.PR_GPU(g, s, g.degree(), 1e-6, 100)
            other[name] = s
        ig.set_option("pr_two_pass", two)
        for name in ("rmat14", "hubby", "er4k", "rmat18"):
            g = graphs[name]
            outs = []
            for _ in range(2):
                s = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
                it, _ = ig.PR_GPU(g, s, g.degree(), 1e-6, 100)
                outs.append(s)
            assert np.array_equal(outs[0], outs[1]), name
            if name in other:
                assert np.array_equal(outs[0], other[name]), name
            ref, _, _ = orc.pr_f64(g, iters=it)
            assert np.abs(outs[0] - ref).sum() / ref.sum() <= PR_TOL, name
    finally:
        ig.set_option("pr_subwarp", old[0])
        ig.set_option("pr_prefetch", old[1])
        ig.set_option("pr_two_pass", old[2])


@pytest.mark.parametrize("pair", [1, 2])
def test_sssp_paired_slices(ig, orc, graphs, pair):
    """Work-item slices expanded two at a time (eight edges per lane, at 3 or
    4 resident blocks per SM): exact distances, with lists of every length
    cut into items (item threshold 4) and with the default threshold."""
    old = {k: ig.get_option(k) for k in ("sssp_pair_slices", "sssp_warp_degree")}
    try:
        ig.set_option("sssp_pair_slices", pair)
        for wd in (64, 4):
            ig.set_option("sssp_warp_degree", wd)
            for name in ("rmat14", "hubby", "road128", "star", "rmat18"):
                g = graphs[name]
                with ig.DeviceCSR(g) as d:
                    for s in (0, g.nodes // 2):
                        dist = np.empty(g.nodes, np.int32)
                        ig.GPUsssp_vertex(int(s), d, dist)
                        assert np.array_equal(dist, orc.sssp(g, int(s))), (name, s, wd)
    finally:
        for k, v in old.items():
            ig.set_option(k, v)


@pytest.mark.parametrize("stage,heavy,pair", [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (1, 0, 1)])
def test_sssp_flag_settling_forms(ig, orc, graphs, stage, heavy, pair):
    """Improved vertices staged per warp and their queue flags settled 32 at
    a time, or settled by the step that found them; with and without the
    light/heavy edge split and the paired slices: exact distances, with most
    lists cut into work items (threshold 4) and with the default threshold."""
    old = {k: ig.get_option(k) for k in ("sssp_stage_flags", "sssp_heavy_split", "sssp_pair_slices",
                                         "sssp_warp_degree")}
    try:
        ig.set_option("sssp_stage_flags", stage)
        ig.set_option("sssp_heavy_split", heavy)
        ig.set_option("sssp_pair_slices", pair)
        for wd in (64, 4):
            ig.set_option("sssp_warp_degree", wd)
            for name in ("rmat14", "hubby", "road128", "star", "rmat18"):
                g = graphs[name]
                with ig.DeviceCSR(g) as d:
                    for s in (0, g.nodes // 2):
                        dist = np.empty(g.nodes, np.int32)
                        ig.GPUsssp_vertex(int(s), d, dist)
                        assert np.array_equal(dist, orc.sssp(g, int(s))), (name, s, wd)
    finally:
        for k, v in old.items():
            ig.set_option(k, v)


@pytest.mark.parametrize("grab", [1, 4, 16])
def test_tc_item_runs(ig, orc, graphs, grab):
    """Block work items taken in runs from a counter instead of a grid
    stride: the same counts, on the plain and the degree-ordered ids."""
    old = (ig.get_option("tc_grab"), ig.get_option("tc_block_chunk"))
    try:
        ig.set_option("tc_grab", grab)
        ig.set_option("tc_block_chunk", 256)  # many items per middle vertex
        for name in ("rmat14", "hubby", "complete", "rmat18"):
            for g in (graphs[name], graphs[name].degree_ordered()):
                with ig.DeviceCSR(g) as d:
                    assert ig.GPUtc_vertex(g.nodes, d.nindex_ptr, d.nlist_ptr)[0] == orc.tc(g), (name, grab)
    finally:
        ig.set_option("tc_grab", old[0])
        ig.set_option("tc_block_chunk", old[1])


@pytest.mark.parametrize("warp_list", [1, 16, 33, 65, 97, 1 << 20])
def test_tc_warp_walk_threshold(ig, orc, graphs, warp_list):
    """Probe lists walked by the whole warp (128, 64 and 32 probes per step)
    from a threshold of one probe up to none at all: the same counts, on the
    plain and the degree-ordered ids, through the block and warp paths."""
    old = ig.get_option("tc_warp_list")
    try:
        ig.set_option("tc_warp_list", warp_list)
        for name in ("rmat14", "hubby", "complete", "star", "rmat18"):
            for g in (graphs[name], graphs[name].degree_ordered()):
                with ig.DeviceCSR(g) as d:
                    assert ig.GPUtc_vertex(g.nodes, d.nindex_ptr, d.nlist_ptr)[0] == orc.tc(g), (name, warp_list)
    finally:
        ig.set_option("tc_warp_list", old)


@pytest.mark.parametrize("pct", [0, 75, 100])
def test_static_share_forms(ig, orc, graphs, pct):
    """Frontier chunks, work-item slice groups (SSSP) and worklist groups
    (MIS) dealt round-robin up to a share of the pass, the rest taken from
    the counter: exact distances and the reference's set, with one- and
    two-slice work items, on the plain and the degree-ordered ids."""
    names = ("sssp_static_pct", "mis_static_pct", "sssp_item_edges", "sssp_warp_degree")
    old = {k: ig.get_option(k) for k in names}
    try:
        ig.set_option("sssp_static_pct", pct)
        ig.set_option("mis_static_pct", pct)
        for ie, wd in ((128, 64), (256, 4)):
            ig.set_option("sssp_item_edges", ie)
            ig.set_option("sssp_warp_degree", wd)
            for name in ("rmat14", "hubby", "road128", "star", "rmat18"):
                for g in (graphs[name], graphs[name].degree_ordered()):
                    with ig.DeviceCSR(g) as d:
                        for s in (0, g.nodes // 2):
                            dist = np.empty(g.nodes, np.int32)
                            ig.GPUsssp_vertex(int(s), d, dist)
                            assert np.array_equal(dist, orc.sssp(g, int(s))), (name, s, ie)
                        st = np.empty(g.nodes, np.int32)
                        ig.GPUmis_vertex(d, None, st)
                        assert np.array_equal(st, orc.mis(g).astype(np.int32)), name
    finally:
        for k, v in old.items():
            ig.set_option(k, v)


def test_pagerank_schedule_independent(ig, orc, graphs):
    """Vertex groups dealt round-robin (100%), partly (75%, 50%) or all from
    the counter (0%): the same scores bit for bit and the same iteration
    count -- each vertex's sum depends only on its list and the residual is
    an exact integer sum -- and within 1e-6 relative L1 of FP64."""
    old = ig.get_option("pr_static_pct")
    try:
        for name in ("rmat14", "hubby", "road128", "rmat18"):
            g = graphs[name]
            outs = []
            for pct in (100, 75, 50, 0):
                ig.set_option("pr_static_pct", pct)
                s = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
                it, _ = ig.PR_GPU(g, s, g.degree(), 1e-6, 100)
                outs.append((it, s))
            for it, s in outs[1:]:
                assert it == outs[0][0] and np.array_equal(s, outs[0][1]), name
            ref, _, _ = orc.pr_f64(g, iters=outs[0][0])
            assert np.abs(outs[0][1] - ref).sum() / ref.sum() <= PR_TOL, name
    finally:
        ig.set_option("pr_static_pct", old)


@pytest.mark.parametrize("claim", [1, 4, 16])
def test_bfs_bottom_up_claims(ig, orc, graphs, claim):
    """Bottom-up levels whose 32-vertex chunks are taken in groups from a
    counter instead of a grid stride: exact levels, bottom-up from the
    first level on (alpha 1) and with the default switch, bitmaps or not."""
    old = {k: ig.get_option(k) for k in ("bfs_bu_claim", "bfs_alpha", "bfs_bitmap")}
    try:
        ig.set_option("bfs_bu_claim", claim)
        for alpha in (1, 14):
            ig.set_option("bfs_alpha", alpha)
            for bitmap in (1, 0):
                ig.set_option("bfs_bitmap", bitmap)
                for name in ("rmat14", "hubby", "road128", "two_grids", "star", "rmat18"):
                    g = graphs[name]
                    r = run_all(ig, g, [0, g.nodes // 2])
                    for k, s in enumerate([0, g.nodes // 2]):
                        assert np.array_equal(r[f"bfs{k}"], orc.bfs(g, s)), (name, s, alpha, bitmap)
                    assert np.array_equal(r["cc"], orc.cc(g)), name
    finally:
        for k, v in old.items():
            ig.set_option(k, v)


@pytest.mark.parametrize("check", [0, 1])
def test_sssp_expanded_check_forms(ig, orc, graphs, check):
    """Queued vertices skipped when their distance has not dropped since
    their last expansion, or expanded again: exact distances either way
    (with and without the degree window, most lists as work items or not)."""
    old = {k: ig.get_option(k) for k in ("sssp_expanded_check", "sssp_window_scale", "sssp_warp_degree")}
    try:
        ig.set_option("sssp_expanded_check", check)
        for ws, wd in ((8, 64), (0, 64), (8, 4)):
            ig.set_option("sssp_window_scale", ws)
            ig.set_option("sssp_warp_degree", wd)
            for name in ("rmat14", "hubby", "road128", "star", "rmat18"):
                g = graphs[name]
                with ig.DeviceCSR(g) as d:
                    for s in (0, g.nodes // 2):
                        dist = np.empty(g.nodes, np.int32)
                        ig.GPUsssp_vertex(int(s), d, dist)
                        assert np.array_equal(dist, orc.sssp(g, int(s))), (name, s, ws, wd)
    finally:
        for k, v in old.items():
            ig.set_option(k, v)


@pytest.mark.parametrize("runs,warp_list", [(1, 64), (1, 1 << 20), (0, 1 << 20), (1, 16)])
def test_tc_short_list_expansion(ig, orc, graphs, runs, warp_list):
    """Short probe lists expanded four consecutive slots per lane (one owner
    search per lane and step) or one owner search per slot, alone or beside
    the whole-warp walks: the same counts on plain and degree-ordered ids."""
    old = {k: ig.get_option(k) for k in ("tc_runs", "tc_warp_list")}
    try:
        ig.set_option("tc_runs", runs)
        ig.set_option("tc_warp_list", warp_list)
        for name in ("rmat14", "hubby", "complete", "star", "grid64", "rmat18"):
            for g in (graphs[name], graphs[name].degree_ordered()):
                with ig.DeviceCSR(g) as d:
                    assert ig.GPUtc_vertex(g.nodes, d.nindex_ptr, d.nlist_ptr)[0] == orc.tc(g), (name, runs)
    finally:
        for k, v in old.items():
            ig.set_option(k, v)


@pytest.mark.parametrize("levels", [1, 2, 5, 32, 0])
def test_cc_truncated_seed_bfs(ig, orc, graphs, levels):
    """The seed BFS of connected components stopped after 1 / 2 / 5 / 32
    levels or run to the end: the vertices beyond it are linked by
    union-find and the min-id labels are exact (high-diameter grids and road
    graphs, skewed graphs, several components)."""
    old = ig.get_option("cc_bfs_levels")
    try:
        ig.set_option("cc_bfs_levels", levels)
        for name in ("road128", "grid64", "two_grids", "rmat14", "hubby", "star", "path", "two_isolated", "rmat18"):
            g = graphs[name]
            lab = np.empty(g.nodes, np.int32)
            with ig.DeviceCSR(g) as d:
                ig.GPUcc_vertex(d, lab)
            assert np.array_equal(lab, orc.cc(g)), (name, levels)
    finally:
        ig.set_option("cc_bfs_levels", old)
