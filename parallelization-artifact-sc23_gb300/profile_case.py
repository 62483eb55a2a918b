"""Small, self-contained workload for Nsight Compute captures: one algorithm
on a synthetic RMAT graph (default scale 21: 2,097,152 vertices, about 63M
directed edges, so the 250 MB neighbour list exceeds the 129 MB L2), run a
few times through the device-resident API.

    python parallelization-artifact-sc23_gb300/profile_case.py --algo bfs [--scale 21 | --graph road:4096]
           [--repeat 3] [--opt sssp_delta=100 ...]

It prints one line per run with the CUDA-event time and the algorithmic
bytes, so a capture can be related to the bench's roofline figures."""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))

import indigo_gb300 as ig  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--algo", choices=["bfs", "sssp", "cc", "mis", "pr", "tc"], required=True)
    ap.add_argument("--scale", type=int, default=21)
    ap.add_argument("--graph", default="", help="instead of --scale: rmat:<scale> | road:<side> | grid:<side>")
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--opt", action="append", default=[], help="kernel option name=value (ig_set_option)")
    args = ap.parse_args()
    for o in args.opt:
        name, value = o.split("=")
        ig.set_option(name, int(value))
    if args.graph:
        kind, _, arg = args.graph.partition(":")
        if kind == "road":  # the high-diameter configuration: 5% of edges deleted, 0.1% shortcuts
            g = ig.road(int(arg), int(arg), 0.05, 0.001, seed=11, maxw=10000)
        elif kind == "grid":
            g = ig.grid2d(int(arg), int(arg), maxw=255)
        else:
            g = ig.rmat(int(arg), 16, seed=7, maxw=1000)
    else:
        g = ig.rmat(args.scale, 16, seed=7, maxw=1000)
    if args.algo == "tc":
        g = g.degree_ordered()
    V, E = g.nodes, g.edges
    src = int(g.pick_sources(1, seed=7)[0])
    with ig.DeviceCSR(g) as d:
        G = ig.DeviceGraph(d)
        out = ig.DeviceBuffer(4 * V)
        cnt = ig.DeviceBuffer(8)
        init = ig.DeviceBuffer.from_array(np.full(V, np.float32(1.0) / np.float32(V), np.float32))
        bytes_per = {"bfs": 4 * (V + 1) + 8 * E + 4 * V, "sssp": 12 * E + 8 * V, "cc": 8 * E + 8 * V,
                     "mis": 8 * E + 12 * V, "pr": 8 * E + 20 * V, "tc": 8 * E + 4 * V}
        a, b = ig.Event(), ig.Event()
        for r in range(args.repeat):
            if args.algo == "pr":
                ig.check(ig.load().ig_memcpy(out.ptr, init.ptr, 4 * V, 3))
            a.record(G.stream)
            if args.algo == "bfs":
                G.bfs(src, out)
            elif args.algo == "sssp":
                G.sssp(src, out)
            elif args.algo == "cc":
                G.cc(out)
            elif args.algo == "mis":
                G.mis(out)
            elif args.algo == "pr":
                G.pagerank(out, 1e-6, 100)
            else:
                G.tc(cnt)
            b.record(G.stream)
            ms = a.elapsed_ms(b)
            info = G.last_run()
            ig.check(info.status)
            mult = max(1, info.iterations) if args.algo == "pr" else 1
            gbs = bytes_per[args.algo] * mult / (ms * 1e-3) / 1e9
            print(f"{args.algo} run {r}: {ms:.3f} ms, iterations {info.iterations}, work {info.work}, "
                  f"aux {list(info.aux)}, "
                  f"{E / (ms * 1e-3) / 1e9:.2f} GTEPS, {gbs:.0f} GB/s algorithmic (V={V}, E={E})")
        G.close()


if __name__ == "__main__":
    main()
