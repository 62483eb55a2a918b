"""Batched form on the GPU: every per-graph result of one batched call equals
the plain single-graph drop-in call on that graph (bit-exact for BFS, CC and
TC; PageRank with the same iteration count and scores within 1e-6 relative L1,
in practice identical), for the first (direct), second (captured into a CUDA
graph) and third (replayed) call."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch(ig, gpu):
    u, vptr = ig.gen_batch(48, vmin=64, vmax=4096, seed=13, maxw=255)
    b = ig.Batch(u, vptr)
    yield b
    b.close()


def plain_results(ig, g):
    with ig.DeviceCSR(g) as d:
        dist = np.empty(g.nodes, np.int32)
        ig.GPUbfs_vertex(0, d, dist)
        lab = np.empty(g.nodes, np.int32)
        ig.GPUcc_vertex(d, lab)
        tc = ig.GPUtc_vertex(g.nodes, d.nindex_ptr, d.nlist_ptr)[0]
    sc = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
    it, _ = ig.PR_GPU(g, sc, g.degree(), 1e-6, 100)
    return dist, lab, tc, sc, it


@pytest.fixture(scope="module")
def expected(ig, batch):
    return [plain_results(ig, ig.unpack(batch.union, batch.vptr, i)) for i in range(batch.graphs)]


def run_batch(ig, b):
    V = b.nodes
    dist = ig.DeviceBuffer(4 * V)
    lab = ig.DeviceBuffer(4 * V)
    cnt = ig.DeviceBuffer(8 * b.graphs)
    init = np.concatenate([np.full(int(b.vptr[i + 1] - b.vptr[i]),
                                   np.float32(1.0) / np.float32(b.vptr[i + 1] - b.vptr[i]), np.float32)
                           for i in range(b.graphs)])
    sc = ig.DeviceBuffer.from_array(init)
    its = ig.DeviceBuffer(4 * b.graphs)
    outs = []
    for call in range(3):  # direct, captured, replayed
        ig.check(ig.load().ig_memcpy(sc.ptr, init.ctypes.data, init.nbytes, 1))
        b.bfs(dist)
        b.cc(lab)
        b.tc(cnt)
        b.pagerank(sc, 1e-6, 100, its)
        info = b.last_run()
        assert info.status == 0
        outs.append((dist.to_array(np.int32, V), lab.to_array(np.int32, V), cnt.to_array(np.uint64, b.graphs),
                     sc.to_array(np.float32, V), its.to_array(np.int32, b.graphs)))
    return outs


def test_batch_equals_plain_calls(ig, batch, expected):
    outs = run_batch(ig, batch)
    for call, (dist, lab, cnt, sc, its) in enumerate(outs):
        for i, (e_dist, e_lab, e_tc, e_sc, e_it) in enumerate(expected):
            v0, v1 = batch.vptr[i], batch.vptr[i + 1]
            assert np.array_equal(dist[v0:v1], e_dist), (call, i, "bfs")
            assert np.array_equal(lab[v0:v1], e_lab), (call, i, "cc")
            assert int(cnt[i]) == e_tc, (call, i, "tc")
            assert int(its[i]) == e_it, (call, i, "pr iterations")
            s = sc[v0:v1].astype(np.float64)
            assert np.abs(s - e_sc).sum() / e_sc.sum() <= 1e-6, (call, i, "pr")


def test_batch_pagerank_bit_identical(ig, batch, expected):
    """With equal iteration counts the per-vertex arithmetic is the same as in
    the single-graph kernel, so the scores are the same bits."""
    dist, lab, cnt, sc, its = run_batch(ig, batch)[-1]
    same = sum(np.array_equal(sc[batch.vptr[i]:batch.vptr[i + 1]], e[3]) for i, e in enumerate(expected))
    assert same == batch.graphs


def test_batch_without_graph_capture(ig, batch, expected):
    batch.use_graphs(False)
    try:
        dist = ig.DeviceBuffer(4 * batch.nodes)
        batch.bfs(dist)
        d = dist.to_array(np.int32, batch.nodes)
    finally:
        batch.use_graphs(True)
    for i, e in enumerate(expected):
        assert np.array_equal(d[batch.vptr[i]:batch.vptr[i + 1]], e[0])


def test_batch_of_tiny_and_edge_case_graphs(ig, gpu):
    from conftest import kat_graphs
    K = kat_graphs(ig)
    gs = [K["single"], K["edge"], K["path"], K["two_isolated"], K["complete"], K["star"], K["two_grids"]]
    u, vptr = ig.pack(gs)
    with ig.Batch(u, vptr) as b:
        dist = ig.DeviceBuffer(4 * u.nodes)
        lab = ig.DeviceBuffer(4 * u.nodes)
        cnt = ig.DeviceBuffer(8 * len(gs))
        b.bfs(dist)
        b.cc(lab)
        b.tc(cnt)
        assert b.last_run().status == 0
        d, l, c = dist.to_array(np.int32, u.nodes), lab.to_array(np.int32, u.nodes), cnt.to_array(np.uint64, len(gs))
    for i, g in enumerate(gs):
        e_dist, e_lab, e_tc, _, _ = plain_results(ig, g)
        assert np.array_equal(d[vptr[i]:vptr[i + 1]], e_dist)
        assert np.array_equal(l[vptr[i]:vptr[i + 1]], e_lab)
        assert int(c[i]) == e_tc


def test_autotune_keeps_results(ig, gpu, expected):
    """Autotuning picks launch variants only: after it, the batch's calls
    (re-captured with the chosen options) give the same results."""
    u, vptr = ig.gen_batch(48, vmin=64, vmax=4096, seed=13, maxw=255)
    with ig.Batch(u, vptr) as b:
        best = b.autotune(("bfs", "cc", "tc", "pr"), reps=1)
        assert set(best) == {"bfs", "cc", "tc", "pr"} and all(v > 0 for v in best.values())
        assert b.get_option("bfs", "blocks_per_sm") in (ig.get_option("blocks_per_sm"), 4, 8)
        assert b.get_option("bfs", "bfs_alpha") in (ig.get_option("bfs_alpha"), 14, 0)
        assert b.get_option("bfs", "bfs_bitmap") in (0, 1)
        assert b.get_option("cc", "hub_degree") in (ig.get_option("hub_degree"), 64, 256, 1024, 4096)
        assert b.get_option("cc", "cc_rounds") in (0, 1)
        assert b.get_option("pr", "pr_hub_degree") in (ig.get_option("pr_hub_degree"), 1024, 4096)
        assert b.get_option("pr", "pr_blocks_per_sm") in (ig.get_option("pr_blocks_per_sm"), 3, 4)
        assert b.get_option("pr", "pr_subwarp") in (0, 1)
        same_pr_form = all(b.get_option("pr", k) == ig.get_option(k) for k in ("pr_subwarp", "pr_two_pass"))
        outs = run_batch(ig, b)
    for call, (dist, lab, cnt, sc, its) in enumerate(outs):
        for i, (e_dist, e_lab, e_tc, e_sc, e_it) in enumerate(expected):
            v0, v1 = b.vptr[i], b.vptr[i + 1]
            assert np.array_equal(dist[v0:v1], e_dist), (call, i, "bfs")
            assert np.array_equal(lab[v0:v1], e_lab), (call, i, "cc")
            assert int(cnt[i]) == e_tc, (call, i, "tc")
            # the tuned PageRank may sum medium lists in another order (sub-warps):
            # within tolerance, and the same bits when it kept the warp form
            s_ = sc[v0:v1].astype(np.float64)
            assert np.abs(s_ - e_sc).sum() / e_sc.sum() <= 1e-6 and abs(int(its[i]) - e_it) <= 1, (call, i, "pr")
            if same_pr_form:
                assert int(its[i]) == e_it and np.array_equal(sc[v0:v1], e_sc), (call, i, "pr bits")


def test_captures_follow_scratch_growth(ig, gpu, expected):
    """BFS and CC are captured into CUDA graphs before the first TC call,
    whose larger buffers make the batch's shared scratch slots grow; the next
    BFS and CC calls must be captured again (their graphs held the old
    addresses) and give the same results."""
    u, vptr = ig.gen_batch(48, vmin=64, vmax=4096, seed=13, maxw=255)
    with ig.Batch(u, vptr) as b:
        V = b.nodes
        dist, lab, cnt = ig.DeviceBuffer(4 * V), ig.DeviceBuffer(4 * V), ig.DeviceBuffer(8 * b.graphs)
        for _ in range(2):  # direct, then captured
            b.bfs(dist)
            b.cc(lab)
        b.tc(cnt)  # first TC call: grows scratch slots BFS and CC use
        for _ in range(2):  # captured again, then replayed
            b.bfs(dist)
            b.cc(lab)
            assert b.last_run().status == 0
            d, l = dist.to_array(np.int32, V), lab.to_array(np.int32, V)
            for i, (e_dist, e_lab, e_tc, _, _) in enumerate(expected):
                v0, v1 = b.vptr[i], b.vptr[i + 1]
                assert np.array_equal(d[v0:v1], e_dist) and np.array_equal(l[v0:v1], e_lab), i
        c = cnt.to_array(np.uint64, b.graphs)
        assert all(int(c[i]) == e[2] for i, e in enumerate(expected))


def test_tuning_database(ig, gpu, expected, tmp_path):
    """autotune(db=...) stores the chosen options under the batch's statistics
    key; a second batch with the same statistics takes them without timing,
    and its results stay those of the plain calls."""
    db = str(tmp_path / "tuning.json")
    u, vptr = ig.gen_batch(48, vmin=64, vmax=4096, seed=13, maxw=255)
    with ig.Batch(u, vptr) as b:
        first = b.autotune(("bfs", "cc", "pr"), reps=1, db=db)
        assert all(v is not None and v > 0 for v in first.values())
        chosen = {a: {n: b.get_option(a, n) for n in ig.Batch.TUNED[a]} for a in ("bfs", "cc", "pr")}
        key = b.stats_key()
    import json
    table = json.load(open(db))
    assert table[key] == chosen
    with ig.Batch(u, vptr) as b2:
        again = b2.autotune(("bfs", "cc", "pr"), reps=1, db=db)
        assert all(v is None for v in again.values())
        assert {a: {n: b2.get_option(a, n) for n in ig.Batch.TUNED[a]} for a in chosen} == chosen
        outs = run_batch(ig, b2)
    dist, lab, cnt, sc, its = outs[-1]
    for i, (e_dist, e_lab, e_tc, e_sc, e_it) in enumerate(expected):
        v0, v1 = vptr[i], vptr[i + 1]
        assert np.array_equal(dist[v0:v1], e_dist) and np.array_equal(lab[v0:v1], e_lab) and int(cnt[i]) == e_tc
        assert abs(int(its[i]) - e_it) <= 1
        assert np.abs(sc[v0:v1].astype(np.float64) - e_sc).sum() / e_sc.sum() <= 1e-6
