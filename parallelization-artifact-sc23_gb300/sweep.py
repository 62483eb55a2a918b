"""Variant sweep: every algorithm under each of its kernel-option variants
(the GB300 counterparts of the suite's style axes), timed on one graph and
written in the layout of the reference's result tables (data/<algo>_cuda.csv:
a "filename" column naming graph, GPU and variant, and a column holding the
throughput in gigaedges per second that the drivers print, E / runtime).

    python parallelization-artifact-sc23_gb300/sweep.py --graph rmat:20 --algos bfs,sssp \
        --out sweep.csv [--repeat 5] [--compare data/bfs_cuda.csv]

Variants differ only in speed: the sweep checks that every variant returns
the same result (bit for bit; PageRank within 1e-6 relative L1 of the first
variant) before it reports a number.  --compare prints, beside each
algorithm's best variant, the best row of a reference table for the same
algorithm (the caller names the file; the reference's graphs are not
generated here, so the comparison is across graphs unless the caller loads
the same .egr)."""
from __future__ import annotations

import argparse
import csv
import itertools
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))

import indigo_gb300 as ig  # noqa: E402

# Option grids per algorithm.  The first entry of every grid is the library
# default, so the first variant is the default configuration.
AXES = {
    "bfs": {"blocks_per_sm": [4, 2, 8], "hub_degree": [256, 64, 1024], "bfs_alpha": [14, 1000000]},
    "sssp": {"blocks_per_sm": [4, 3], "sssp_item_edges": [256, 512], "sssp_window_scale": [8, 4, 0],
             "sssp_window_degree": [16, 64], "sssp_delta_scale": [128, 32], "sssp_heavy_split": [0, 1]},
    "cc": {"blocks_per_sm": [4, 8], "hub_degree": [256, 64, 4096]},
    "mis": {"blocks_per_sm": [4, 2, 8]},
    "pr": {"pr_blocks_per_sm": [4, 3, 2], "pr_hub_degree": [1024, 256, 4096], "pr_chunk": [4096, 512]},
    "tc": {"tc_block_chunk": [4096, 1024]},
}
# short labels for the variant names (like the suite's style words)
LABEL = {"blocks_per_sm": "B", "hub_degree": "Hub", "bfs_alpha": "Alpha", "sssp_item_edges": "Item",
         "sssp_warp_degree": "Warp", "sssp_window_scale": "Win", "sssp_window_degree": "WinDeg",
         "sssp_delta_scale": "Delta", "sssp_heavy_split": "Split", "pr_blocks_per_sm": "B",
         "pr_hub_degree": "Hub", "pr_chunk": "Chunk", "tc_block_chunk": "Item"}


def variants(algo: str) -> list:
    """All option combinations of an algorithm's grid, default first."""
    axes = AXES[algo]
    names = list(axes)
    return [dict(zip(names, combo)) for combo in itertools.product(*(axes[n] for n in names))]


def variant_name(graph: str, algo: str, opts: dict) -> str:
    style = "_".join(f"{LABEL[k]}{v}" for k, v in opts.items())
    return f"{graph}_gb300_{algo.upper()}_GB300_{style}.cu"


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


def sweep(g, algos, repeat: int, graph_name: str, log=print) -> dict:
    gd = g.degree_ordered() if "tc" in algos else None
    src = int(g.pick_sources(1, seed=7)[0])
    names = ("blocks_per_sm", "hub_degree", "bfs_alpha", "sssp_item_edges", "sssp_warp_degree", "sssp_window_scale",
             "sssp_window_degree", "sssp_delta_scale", "sssp_heavy_split", "pr_blocks_per_sm", "pr_hub_degree",
             "pr_chunk", "tc_block_chunk")
    saved = {k: ig.get_option(k) for k in names}
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
                for opts in variants(algo):
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
                    if first is None:
                        first = r
                    elif algo == "pr":
                        rel = np.abs(r - first).sum() / np.abs(first).sum()
                        if rel > 1e-6:
                            raise RuntimeError(f"{algo} variant {opts}: relative L1 {rel} from the first variant")
                    elif not np.array_equal(r, first):
                        raise RuntimeError(f"{algo} variant {opts} changed the result")
                    ms = float(np.median(times))
                    gteps = (gd.edges if algo == "tc" else g.edges) / (ms * 1e-3) / 1e9
                    rows[algo].append((variant_name(graph_name, algo, opts), gteps))
                    log(f"{algo} {opts}: median {ms:.3f} ms, {gteps:.3f} gigaedges/s")
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
        if a not in AXES:
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
