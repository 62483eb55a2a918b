"""Variant sweep over the suite's style axes: every algorithm under each
combination of its axes -- the GB300 counterparts of the paper's vertex /
edge parallel, push / pull, data- / topology-driven and thread / warp /
block granularity choices -- timed on one graph and written in the layout of
the reference's result tables (data/<algo>_cuda.csv: a "filename" column
naming graph, GPU and variant, and a column holding the throughput in
gigaedges per second that the drivers print, E / runtime).

    python parallelization-artifact-sc23_gb300/sweep.py --graph rmat:20 --algos bfs,sssp \
        --out sweep.csv [--repeat 5] [--compare data/bfs_cuda.csv]

Variants differ only in speed: the sweep checks that every variant returns
the same result (bit for bit; PageRank within 1e-6 relative L1 of the first
variant) before it reports a number (the GPU tests check every variant
against the oracle instead).  --compare prints, beside each algorithm's best
variant, the best row of a reference table for the same algorithm (the
caller names the file; the reference's graphs are not generated here, so the
comparison is across graphs unless the caller loads the same .egr)."""
from __future__ import annotations

import argparse
import csv
import itertools
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))

import indigo_gb300 as ig  # noqa: E402

BIG = 1 << 30
# Style axes per algorithm: axis -> {style word: kernel options}.  The first
# word of every axis is the library default, so the first variant is the
# default configuration.  Words follow the suite's file names (V / E, Push /
# Pull, Data / Topo, Thread / Warp / Block) where the GB300 design has the
# counterpart:
#   BFS  direction: PushPull = direction-optimising (data-driven top-down
#        worklist levels, topology-driven bottom-up levels), Push = top-down
#        only (Data), Pull = bottom-up as soon as the frontier has edges,
#        back to top-down only for the small last levels (Topo);
#        granularity: lists expanded by the warp's lanes, every list above
#        32 spread over the whole grid (Grid, the default), only lists above
#        256 (WarpGrid), or warp only; Bitmap / Dist: how a pull level tests
#        a neighbour.
#   SSSP parallel: V = each vertex's list expanded by the warp that holds it,
#        E = every list cut into edge work items, VE = lists above 64 edges as
#        work items (default); order: Window = long lists expanded near
#        Dijkstra order, NoWindow; sync: Sync2 = work items after a second
#        grid barrier per round, Sync1 = within the round (one barrier);
#        Plain / LightHeavy edge split; flags: Staged = improved vertices'
#        queue flags settled 32 at a time, Immediate = by the step that found
#        them; schedule: Static75 = the first 75% of a pass's chunks dealt
#        round-robin, Dynamic = all but the first per warp from a counter.
#        (Always a data-driven worklist.)
#   CC   link: BfsSeed = the largest-degree vertex's component labelled by
#        a BFS from it (direction-optimising traversal), union-find for the
#        rest; Pass = neighbour sampling (two neighbours linked in one pass
#        with path halving), Rounds = one round per sampled neighbour with a
#        compression after each, FlatPass = Pass after flattening the initial
#        forest; granularity as BFS.  (Hooking pushes along edges.)
#   MIS  residency (B4 / B2 / B8 blocks per SM); schedule: Dynamic worklist
#        groups from a counter, Static75 = 75% dealt round-robin.
#   PR   gather: OnePass = contributions gathered while summing, TwoPass =
#        every edge's contribution gathered first in one dense pass (measured
#        slower: the gathers cost the same either way); granularity: SubWarp
#        = medium lists four at a time by 8-lane sub-warps, WarpPair = by the
#        whole warp two at a time; hub chunks of 1024 / 4096 / 256 edges;
#        NoPrefetch / Prefetch of each warp's next lists into L2.
#        (Pull only: push PageRank needs float atomics, not deterministic.)
#   TC   block work items of 4096 / 1024 in-neighbours, taken by blocks in
#        runs of 2 or 4 from a counter or dealt in a grid stride; walk: probe
#        lists from 64 (Walk64) or 96 (Walk96) probes walked by the whole
#        warp, or every list through the owner search (Owner).
STYLES = {
    "bfs": {"direction": {"PushPull": {}, "Push": {"bfs_alpha": 0}, "Pull": {"bfs_alpha": 1000000}},
            "granularity": {"Grid": {}, "WarpGrid": {"bfs_hub_degree": 256}, "Warp": {"bfs_hub_degree": BIG}},
            "test": {"Bitmap": {}, "Dist": {"bfs_bitmap": 0}}},
    "sssp": {"parallel": {"VE": {}, "V": {"sssp_warp_degree": BIG}, "E": {"sssp_warp_degree": 1}},
             "order": {"Window": {}, "NoWindow": {"sssp_window_scale": 0}},
             "sync": {"Sync2": {}, "Sync1": {"sssp_merge_below": BIG}},
             "split": {"Plain": {}, "LightHeavy": {"sssp_heavy_split": 1}},
             "flags": {"Staged": {}, "Immediate": {"sssp_stage_flags": 0}},
             "schedule": {"Static75": {}, "Dynamic": {"sssp_static_pct": 0}}},
    "cc": {"link": {"BfsSeed": {}, "Pass": {"cc_bfs_seed": 0}, "Rounds": {"cc_bfs_seed": 0, "cc_rounds": 1},
                    "FlatPass": {"cc_bfs_seed": 0, "cc_rounds": 2}},
           "granularity": {"WarpGrid": {}, "Grid": {"hub_degree": 64}, "Warp": {"hub_degree": BIG}}},
    "mis": {"residency": {"B4": {}, "B2": {"blocks_per_sm": 2}, "B8": {"blocks_per_sm": 8}},
            "schedule": {"Dynamic": {}, "Static75": {"mis_static_pct": 75}}},
    "pr": {"gather": {"OnePass": {}, "TwoPass": {"pr_two_pass": 1}},
           "granularity": {"SubWarp": {}, "WarpPair": {"pr_subwarp": 0}},
           "hubs": {"Chunk1024": {}, "Chunk4096": {"pr_hub_degree": 4096}, "Chunk256": {"pr_hub_degree": 256}},
           "prefetch": {"NoPrefetch": {}, "Prefetch": {"pr_prefetch": 1}}},
    "tc": {"items": {"Item4096": {}, "Item1024": {"tc_block_chunk": 1024}},
           "schedule": {"Runs2": {}, "Stride": {"tc_grab": 0}, "Runs4": {"tc_grab": 4}},
           "walk": {"Walk64": {}, "Walk96": {"tc_warp_list": 96}, "Owner": {"tc_warp_list": 1 << 20}}},
}
AXES = STYLES  # the per-algorithm axes (name kept for callers)
OPTION_NAMES = sorted({k for axes in STYLES.values() for words in axes.values() for o in words.values() for k in o})


def variants(algo: str) -> list:
    """All style combinations of an algorithm, default first: a list of
    (style words, kernel options)."""
    axes = STYLES[algo]
    out = []
    for combo in itertools.product(*(list(axes[a].items()) for a in axes)):
        words = [w for w, _ in combo]
        opts = {}
        for _, o in combo:
            opts.update(o)
        out.append((words, opts))
    return out


def variant_name(graph: str, algo: str, words: list) -> str:
    return f"{graph}_gb300_{algo.upper()}_GB300_{'_'.join(words)}.cu"


def write_csv(path: str, algo_rows: dict) -> None:
    """algo_rows: {algo: [(name, gteps), ...]} -> one two-column table per
    algorithm, concatenated, in the reference's quoting."""
    with open(path, "w", newline="") as f:
        w = csv.writer(f, quoting=csv.QUOTE_ALL)
        for algo, rows in algo_rows.items():
            w.writerow(["filename", algo])
            for name, gteps in rows:
                w.writerow([name + "\n", f"{gteps:.6f}"])


def read_reference_csv(path: str) -> list:
    """[(filename, throughput)] of a reference result table."""
    out = []
    with open(path, newline="") as f:
        r = csv.reader(f)
        next(r, None)
        for row in r:
            if len(row) >= 2:
                try:
                    out.append((row[0].strip(), float(row[1])))
                except ValueError:
                    pass
    return out


def load_graph(spec: str):
    kind, _, arg = spec.partition(":")
    if kind == "rmat":
        return ig.rmat(int(arg or 20), 16, seed=7, maxw=1000)
    if kind == "road":
        n = int(arg or 1024)
        return ig.road(n, n, 0.05, 0.001, seed=11, maxw=10000)
    if kind == "grid":
        n = int(arg or 256)
        return ig.grid2d(n, n, maxw=255)
    if kind == "egr":
        return ig.read_egr(arg)
    raise ValueError(f"unknown graph spec {spec}")


def run_algo(algo, G, GT, g, out, scores, cnt, src):
    if algo == "bfs":
        G.bfs(src, out)
    elif algo == "sssp":
        G.sssp(src, out)
    elif algo == "cc":
        G.cc(out)
    elif algo == "mis":
        G.mis(out)
    elif algo == "pr":
        init = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), np.float32)
        ig.check(ig.load().ig_memcpy(scores.ptr, init.ctypes.data, init.nbytes, 1))
        G.pagerank(scores, 1e-6, 100)
    else:
        GT.tc(cnt)


def result(algo, g, out, scores, cnt):
    if algo == "pr":
        return scores.to_array(np.float32, g.nodes).astype(np.float64)
    if algo == "tc":
        return cnt.to_array(np.uint64, 1)
    return out.to_array(np.int32, g.nodes)


def sweep(g, algos, repeat: int, graph_name: str, log=print, check=None) -> dict:
    """Runs every variant of every algorithm; returns {algo: [(name, gteps)]}.
    check(algo, words, result, iterations, graph) validates each variant's
    result (default: equal to the first variant's; PageRank within 1e-6)."""
    gd = g.degree_ordered() if "tc" in algos else None
    src = int(g.pick_sources(1, seed=7)[0])
    saved = {k: ig.get_option(k) for k in OPTION_NAMES + ["bfs_beta"]}
    rows = {}
    with ig.DeviceCSR(g) as d:
        dd = ig.DeviceCSR(gd) if gd is not None else None
        G = ig.DeviceGraph(d)
        GT = ig.DeviceGraph(dd) if dd is not None else None
        out, scores, cnt = ig.DeviceBuffer(4 * g.nodes), ig.DeviceBuffer(4 * g.nodes), ig.DeviceBuffer(8)
        a, b = ig.Event(), ig.Event()
        try:
            for algo in algos:
                first = None
                rows[algo] = []
                for words, opts in variants(algo):
                    for k, v in saved.items():
                        ig.set_option(k, v)
                    for k, v in opts.items():
                        ig.set_option(k, v)
                    run_algo(algo, G, GT, g, out, scores, cnt, src)  # warm-up
                    stream = (GT if algo == "tc" else G).stream  # events on the stream that runs it
                    times = []
                    for _ in range(repeat):
                        a.record(stream)
                        run_algo(algo, G, GT, g, out, scores, cnt, src)
                        b.record(stream)
                        times.append(a.elapsed_ms(b))
                    info = (GT if algo == "tc" else G).last_run()
                    ig.check(info.status)
                    r = result(algo, g, out, scores, cnt)
                    if check is not None:
                        check(algo, words, r, info.iterations, gd if algo == "tc" else g, src)
                    elif first is None:
                        first = r
                    elif algo == "pr":
                        rel = np.abs(r - first).sum() / np.abs(first).sum()
                        if rel > 1e-6:
                            raise RuntimeError(f"{algo} variant {words}: relative L1 {rel} from the first variant")
                    elif not np.array_equal(r, first):
                        raise RuntimeError(f"{algo} variant {words} changed the result")
                    ms = float(np.median(times))
                    gteps = (gd.edges if algo == "tc" else g.edges) / (ms * 1e-3) / 1e9
                    rows[algo].append((variant_name(graph_name, algo, words), gteps))
                    log(f"{algo} {'_'.join(words)}: median {ms:.3f} ms, {gteps:.3f} gigaedges/s")
        finally:
            for k, v in saved.items():
                ig.set_option(k, v)
            G.close()
            if GT is not None:
                GT.close()
            if dd is not None:
                dd.close()
    return rows


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--graph", default="rmat:20", help="rmat:<scale> | road:<side> | grid:<side> | egr:<path>")
    ap.add_argument("--algos", default="bfs,sssp,cc,mis,pr,tc")
    ap.add_argument("--repeat", type=int, default=5)
    ap.add_argument("--out", default="sweep.csv")
    ap.add_argument("--compare", action="append", default=[], help="a reference result table to compare with")
    args = ap.parse_args()
    algos = [a for a in args.algos.split(",") if a]
    for a in algos:
        if a not in STYLES:
            raise SystemExit(f"unknown algorithm {a}")
    g = load_graph(args.graph)
    name = args.graph.replace(":", "").replace("/", "_")
    rows = sweep(g, algos, args.repeat, name)
    write_csv(args.out, rows)
    for algo, r in rows.items():
        best = max(r, key=lambda t: t[1])
        print(f"best {algo}: {best[1]:.3f} gigaedges/s  {best[0]}")
    for path in args.compare:
        ref = read_reference_csv(path)
        if ref:
            top = max(ref, key=lambda t: t[1])
            print(f"{path}: best published {top[1]:.3f} gigaedges/s  {top[0]}")


if __name__ == "__main__":
    main()
