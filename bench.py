#!/usr/bin/env python3
"""Benchmark of the Indigo2 hot path on one GB300 (or N replicas).

Workload (one "step"): the six algorithms on the synthetic RMAT scale-22 graph
(4,194,304 vertices, edge factor 16, a/b/c/d = .57/.19/.19/.05, seed 7, vertex
ids permuted, self loops and duplicates removed, symmetrised, int32 weights in
[1, 1000]): BFS and SSSP from each of 16 sources, CC, MIS, PageRank (FP32,
d = 0.85, L1 residual 1e-6, <= 100 iterations) and triangle counting on the
degree-ordered copy of the graph.

Metric: GTEPS over the step, the reference's definition (g.edges / runtime,
include/sssp_vertex_cuda.h:167) summed over the step's 36 runs:
value = 36 * E / step time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl ours` (default) prints one JSON line with the device-resident value,
the end-to-end value through the reference-facing C ABI with host buffers,
the roofline of the dominant kernel and the CPU baseline.  `--impl reference`
times the reference's own best-published C++ variants (built from its staged
sources into oracle/_ref; the oracle's threaded restatement of them where
they are not built) on the host cores for the same workload, every step the
full workload, and loads no GPU library.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "parallelization-artifact-sc23_gb300"))
sys.path.insert(0, str(ROOT))

SCALE, EDGE_FACTOR, RMAT_ABC, SEED, MAXW = 22, 16, (0.57, 0.19, 0.19), 7, 1000
N_SOURCES = 16
PR_EPS, PR_MAX_ITER = 1e-6, 100
RUNS_PER_STEP = 2 * N_SOURCES + 4
METRIC = "GTEPS (RMAT-22: 16x BFS + 16x SSSP + CC + MIS + PR + TC)"
UNIT = "GTEPS"
ALGOS = ["bfs", "sssp", "cc", "mis", "pr", "tc"]


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- dist
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        return self._reduce(x, "MAX")

    def sum(self, x: float) -> float:
        return self._reduce(x, "SUM")

    def _reduce(self, x: float, op: str) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=getattr(self.td.ReduceOp, op))
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


# ----------------------------------------------------------------------------- graph
def make_workload(ig):
    t0 = time.time()
    g = ig.rmat(SCALE, EDGE_FACTOR, *RMAT_ABC, seed=SEED, maxw=MAXW, permute=True)
    gd = g.degree_ordered()
    sources = g.pick_sources(N_SOURCES, seed=SEED)
    log(f"[bench] RMAT-{SCALE}: V={g.nodes} E={g.edges} generated in {time.time() - t0:.1f}s")
    return g, gd, sources


def algorithmic_bytes(g, gd, pr_iters: int) -> dict:
    """Bytes each algorithm must move once (4-byte words, each logical access
    counted once): BFS 4(V+1)+8E+4V, SSSP 12E+8V, CC 8E+8V, MIS 8E+12V,
    PR iters*(8E+20V), TC sum over oriented edges u->v of 4(d+(u)+d+(v)) + 4E + 4V."""
    V, E = g.nodes, g.edges
    deg = gd.degree().astype(np.int64)
    # degree-ordered ids: the oriented out-degree is the count of neighbours with a larger id
    src = np.repeat(np.arange(gd.nodes, dtype=np.int64), deg)
    up = gd.nlist.astype(np.int64) > src
    dplus = np.bincount(src[up], minlength=gd.nodes).astype(np.int64)
    tc = 4 * int((dplus[src[up]] + dplus[gd.nlist[up]]).sum()) + 4 * E + 4 * V
    return {
        "bfs": 4 * (V + 1) + 8 * E + 4 * V,
        "sssp": 12 * E + 8 * V,
        "cc": 8 * E + 8 * V,
        "mis": 8 * E + 12 * V,
        "pr": max(1, pr_iters) * (8 * E + 20 * V),
        "tc": tc,
    }


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, val in zip(names, r[5:9]):
                if val.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- ours
def run_ours(args, dist: Dist):
    import indigo_gb300 as ig

    ig.check(ig.load().ig_set_device(dist.local))
    g, gd, sources = make_workload(ig)
    V, E = g.nodes, g.edges

    d = ig.DeviceCSR(g)
    dd = ig.DeviceCSR(gd)
    stream = ig.create_stream()
    G = ig.DeviceGraph(d)
    GT = ig.DeviceGraph(dd)
    G.set_stream(stream)
    GT.set_stream(stream)
    dist_buf = ig.DeviceBuffer(4 * V)
    lab = ig.DeviceBuffer(4 * V)
    st = ig.DeviceBuffer(4 * V)
    init = np.full(V, np.float32(1.0) / np.float32(V), np.float32)
    scores0 = ig.DeviceBuffer.from_array(init)
    scores = ig.DeviceBuffer(4 * V)
    count = ig.DeviceBuffer(8)
    L = ig.load()
    calls = {"bfs": N_SOURCES, "sssp": N_SOURCES, "cc": 1, "mis": 1, "pr": 1, "tc": 1}
    ev = {k: [(ig.Event(), ig.Event()) for _ in range(calls[k])] for k in ALGOS}
    acc = {k: 0.0 for k in ALGOS}
    call_ms = {k: [] for k in ALGOS}  # every timed call, for median and range

    def timed_call(k, i, fn):
        ev[k][i][0].record(stream)
        fn()
        ev[k][i][1].record(stream)

    def step(timed: bool):
        for i, s in enumerate(sources):
            timed_call("bfs", i, lambda: G.bfs(int(s), dist_buf))
        for i, s in enumerate(sources):
            timed_call("sssp", i, lambda: G.sssp(int(s), dist_buf))
        timed_call("cc", 0, lambda: G.cc(lab))
        timed_call("mis", 0, lambda: G.mis(st))
        # the score reset is part of the PageRank call's time
        timed_call("pr", 0, lambda: (ig.check(L.ig_memcpy_async(scores.ptr, scores0.ptr, 4 * V, 3, stream)),
                                     G.pagerank(scores, PR_EPS, PR_MAX_ITER)))
        timed_call("tc", 0, lambda: GT.tc(count))
        if timed:
            for k in ALGOS:
                for a, b in ev[k]:
                    ms = a.elapsed_ms(b)
                    acc[k] += ms
                    call_ms[k].append(ms)

    # warm-up (untimed), then validate the outputs of one step
    for _ in range(args.warmup):
        step(False)
    G.synchronize()
    info_g, info_t = G.last_run(), GT.last_run()
    if info_g.status or info_t.status:
        raise RuntimeError(f"device run failed: status {info_g.status} / {info_t.status}")
    pr_iters = info_g.iterations
    validation = validate(ig, g, G, GT, sources, dist_buf, lab, st, scores, count)

    t_start, t_end = ig.Event(), ig.Event()
    launches0 = ig.kernel_launches()
    clocks = ClockSampler(dist.local)
    dist.barrier()
    ig.check(L.ig_stream_synchronize(stream))
    t_start.record(stream)
    for _ in range(args.steps):
        step(True)
    t_end.record(stream)
    ig.check(L.ig_stream_synchronize(stream))
    dist.barrier()
    clk = clocks.stop()
    ms_total = t_start.elapsed_ms(t_end)
    launches = ig.kernel_launches() - launches0
    if G.last_run().status or GT.last_run().status:
        raise RuntimeError("device error during the timed steps")
    ms_max = dist.max(ms_total)
    ms_per_step = ms_max / args.steps
    value = dist.world * RUNS_PER_STEP * E / (ms_per_step * 1e-3) / 1e9

    # per-algorithm numbers and the roofline of the dominant kernel
    peaks = load_peaks()
    abytes = algorithmic_bytes(g, gd, pr_iters)
    per = {}
    for k in ALGOS:
        ms_call = acc[k] / args.steps / calls[k]
        gbs = abytes[k] / (ms_call * 1e-3) / 1e9
        cm = np.array(call_ms[k])
        per[k] = {"ms_per_call": round(ms_call, 4), "calls_timed": int(cm.size),
                  "median_ms": round(float(np.median(cm)), 4), "min_ms": round(float(cm.min()), 4),
                  "max_ms": round(float(cm.max()), 4), "gteps": round(E / (ms_call * 1e-3) / 1e9, 3),
                  "algorithmic_bytes": abytes[k], "achieved_gbs": round(gbs, 1),
                  "hbm_frac": round(gbs / peaks["hbm_gbs"], 4)}
        if k in DRAM_BYTES_PER_CALL:  # what DRAM actually moved (capture, scaled), per unit of this call's time
            dg = DRAM_BYTES_PER_CALL[k] / (ms_call * 1e-3) / 1e9
            per[k].update({"dram_bytes_per_call": DRAM_BYTES_PER_CALL[k], "dram_gbs": round(dg, 1),
                           "dram_frac": round(dg / peaks["hbm_gbs"], 4)})
    # The triangle-count formula counts every intersection read once, but the
    # exact-bitmap kernel serves one side of each probe from shared memory:
    # its "achieved" can exceed the copy peak.  dram_frac is the DRAM figure.
    per["tc"]["hbm_frac_note"] = ("algorithmic bytes count probe reads served from shared memory; "
                                  "dram_frac is what DRAM moved")
    per["pr"]["iterations"] = pr_iters
    shares = {k: acc[k] / max(1e-9, sum(acc.values())) for k in ALGOS}
    dom = max(shares, key=shares.get)
    traffic = DRAM_BYTES_PER_CALL.get(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": per[dom]["achieved_gbs"], "peak": peaks["hbm_gbs"],
                "peak_source": peaks["source"], "unit": "GB/s",
                "frac": round(per[dom]["achieved_gbs"] / peaks["hbm_gbs"], 4), "traffic": traffic,
                "algorithmic_bytes_per_launch": abytes[dom], "share_of_step": round(shares[dom], 4),
                "timing": "CUDA events around each call on the launching stream, averaged over the timed steps"}

    # Random-access ceiling: SSSP and PageRank are bound by data-dependent
    # 4-byte reads of per-vertex arrays (one 32-byte sector each), so they are
    # also reported against the device's measured rate of such reads.
    gps = ig.probe_random_gather(V, 1 << 29, 3)
    relaxed = []
    for s in sources:  # edges expanded per SSSP call (one random distance read each)
        G.sssp(int(s), dist_buf)
        relaxed.append(G.last_run().aux[2])
    sssp_rate = float(np.mean(relaxed)) / (per["sssp"]["ms_per_call"] * 1e-3)
    pr_rate = E * pr_iters / (per["pr"]["ms_per_call"] * 1e-3)
    random_access = {"unit": "random 4-byte reads/s", "peak": round(gps, -6),
                     "peak_source": "measured now: ig_probe_random_gather, V-float table (L2-resident), 8 reads "
                                    "in flight per thread",
                     "sssp_reads_per_call": int(np.mean(relaxed)), "sssp": round(sssp_rate, -6),
                     "sssp_frac": round(sssp_rate / gps, 4), "pr_reads_per_call": int(E * pr_iters),
                     "pr": round(pr_rate, -6), "pr_frac": round(pr_rate / gps, 4)}

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(ig, g, gd, sources, args, dist)

    cpu = None
    if dist.world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(g, gd, sources, validation)
        per["pr"].update(pagerank_error(g, scores.to_array(np.float32, V), pr_iters))

    for h in (G, GT):
        h.close()
    d.close()
    dd.close()
    forms = None
    if not args.no_forms:
        bt = run_batched(args, dist)
        sv = run_served(args, dist)
        forms = {
            "batched": {k: bt[k] for k in ("metric", "value", "unit", "ms_per_step", "scaling", "config",
                                           "per_algo_ms", "pr_iterations_per_graph", "autotuned", "plain",
                                           "speedup_vs_plain", "clocks", "gpu_launches")},
            "served": {k: sv[k] for k in ("metric", "value", "unit", "config", "per_kind", "clocks")},
        }
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32/f32", "data": "synthetic",
        "config": {"workload": f"rmat{SCALE}_ef{EDGE_FACTOR}_six_algorithms", "vertices": V, "edges": E,
                   "rmat_abcd": [0.57, 0.19, 0.19, 0.05], "seed": SEED, "weights": f"[1,{MAXW}]",
                   "sources": N_SOURCES, "pr_epsilon": PR_EPS, "pr_max_iter": PR_MAX_ITER,
                   "tc_input": "degree-ordered relabelling", "runs_per_step": RUNS_PER_STEP,
                   "l2": "inputs larger than L2 (nlist+eweight %.0f MB > 129 MB)" % (8 * E / 1e6),
                   "parallelism": "replicas" if dist.world > 1 else "single GPU"},
        "e2e": e2e, "roofline": roofline, "random_access": random_access, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
        "per_algo": per, "validation": validation, "forms": forms,
    }
    return out


def run_e2e(ig, g, gd, sources, args, dist: Dist):
    """Same step through the drop-in C ABI (reference pointer residency) with
    the graph copied from pinned host memory every step and every result read
    back to pinned host memory.  The copies of a step's inputs run on their
    own stream and overlap work that does not read them: the degree-ordered
    graph (TC's input) loads during BFS and SSSP, and the next step's graph
    loads during TC (not during PageRank, whose drop-in call uploads its own
    copy of the graph and would share the host-to-device bandwidth with it).
    Every step still copies all of its inputs inside the timed region."""
    import ctypes
    L = ig.load()
    V, E = g.nodes, g.edges

    def pinned(nbytes):
        p = ctypes.c_void_p()
        ig.check(L.ig_host_alloc_pinned(ctypes.byref(p), max(1, nbytes)))
        return p.value

    def pinned_copy(a: np.ndarray):
        p = pinned(a.nbytes)
        ctypes.memmove(p, a.ctypes.data, a.nbytes)
        return p

    hp = {"ni": pinned_copy(g.nindex), "nl": pinned_copy(g.nlist), "ew": pinned_copy(g.eweight),
          "dni": pinned_copy(gd.nindex), "dnl": pinned_copy(gd.nlist), "deg": pinned_copy(g.degree())}
    init = np.full(V, np.float32(1.0) / np.float32(V), np.float32)
    h_scores = pinned(4 * V)
    h_out = pinned(4 * V)
    d = ig.DeviceCSR(g)    # device arrays reused; refilled from pinned memory each step
    dd = ig.DeviceCSR(gd)
    hc = ig.CSR()
    hc.nodes, hc.edges = V, E
    ip = ctypes.POINTER(ctypes.c_int)
    hc.nindex, hc.nlist, hc.eweight = ctypes.cast(hp["ni"], ip), ctypes.cast(hp["nl"], ip), ip()
    t = ctypes.c_double()
    cnt = ctypes.c_longlong()
    it = ctypes.c_int()
    h2d = 4 * (V + 1) + 8 * E + 4 * (V + 1) + 4 * E
    d2h = 4 * V * (2 * N_SOURCES + 2) + 8 + 4 * V
    h2d += 4 * (V + 1) + 4 * E + 4 * V + 4 * V  # PR_GPU uploads nindex, nlist, degree, scores itself

    h = ctypes.c_void_p()
    ig.check(L.ig_stream_create_nonblocking(ctypes.byref(h)))
    cs = h.value  # copy stream, not ordered with the drop-ins' result copies

    def upload(dst, src, nbytes):
        ig.check(L.ig_memcpy_async(ctypes.cast(dst, ctypes.c_void_p), src, nbytes, 1, cs))

    def upload_graph():
        upload(d.c.nindex, hp["ni"], 4 * (V + 1))
        upload(d.c.nlist, hp["nl"], 4 * E)
        upload(d.c.eweight, hp["ew"], 4 * E)

    def upload_tc_graph():
        upload(dd.c.nindex, hp["dni"], 4 * (V + 1))
        upload(dd.c.nlist, hp["dnl"], 4 * E)

    def step(last: bool):
        ig.check(L.ig_stream_synchronize(cs))  # this step's graph is resident
        upload_tc_graph()
        for s in sources:
            ig.check(L.ig_bfs_vertex(int(s), ctypes.byref(d.c), h_out, ctypes.byref(t)))
        for s in sources:
            ig.check(L.ig_sssp_vertex(int(s), ctypes.byref(d.c), h_out, ctypes.byref(t)))
        ig.check(L.ig_cc_vertex(ctypes.byref(d.c), h_out, ctypes.byref(t)))
        ig.check(L.ig_mis_vertex(ctypes.byref(d.c), None, h_out, ctypes.byref(t)))
        ctypes.memmove(h_scores, init.ctypes.data, 4 * V)
        ig.check(L.ig_pr(ctypes.byref(hc), h_scores, hp["deg"], PR_EPS, PR_MAX_ITER, ctypes.byref(it),
                         ctypes.byref(t)))
        ig.check(L.ig_stream_synchronize(cs))  # the TC graph is resident
        if not last:
            upload_graph()  # next step's graph, overlapping TC (MIS was its last reader)
        ig.check(L.ig_tc_vertex(ctypes.byref(cnt), V, ctypes.cast(dd.c.nindex, ctypes.c_void_p),
                                ctypes.cast(dd.c.nlist, ctypes.c_void_p), ctypes.byref(t)))

    for _ in range(max(1, args.warmup)):
        upload_graph()
        step(True)
    ig.check(L.ig_device_synchronize())
    dist.barrier()
    t0 = time.perf_counter()
    upload_graph()  # the first step's graph
    for i in range(args.steps):
        step(i == args.steps - 1)
    ig.check(L.ig_device_synchronize())
    el = time.perf_counter() - t0
    el = dist.max(el)
    d.close()
    dd.close()
    ig.check(L.ig_stream_destroy(cs))
    for p in list(hp.values()) + [h_scores, h_out]:
        L.ig_host_free_pinned(p)
    value = dist.world * RUNS_PER_STEP * E * args.steps / el / 1e9
    return {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": round(1e3 * el / args.steps, 3),
            "api": "drop-in C ABI (ig_bfs_vertex ... ig_tc_vertex), host wall clock, pinned host buffers"}


def validate(ig, g, G, GT, sources, dist_buf, lab, st, scores, count) -> dict:
    """Size-independent properties of one step's results (numpy, untimed)."""
    V = g.nodes
    src = np.repeat(np.arange(V, dtype=np.int64), g.degree())
    nl = g.nlist.astype(np.int64)
    INF = 2147483647
    s0 = int(sources[0])
    G.bfs(s0, dist_buf)
    dd = dist_buf.to_array(np.int32, V).astype(np.int64)
    reach = dd < INF
    ok_bfs = dd[s0] == 0 and bool(np.all(np.abs(dd[src] - dd[nl])[reach[src]] <= 1)) and \
        bool(np.all(reach[src] == reach[nl]))
    G.sssp(s0, dist_buf)
    ds = dist_buf.to_array(np.int32, V).astype(np.int64)
    w = g.eweight.astype(np.int64)
    r = ds[src] < INF
    ok_sssp = ds[s0] == 0 and bool(np.all(ds[nl][r] <= ds[src][r] + w[r]))
    # tightness: every reached vertex but the source has a neighbour on a shortest path
    tight = np.zeros(V, bool)
    hit = r & (ds[nl] == ds[src] + w)
    tight[nl[hit]] = True
    tight[s0] = True
    ok_sssp = ok_sssp and bool(np.all(tight[ds < INF]))
    G.cc(lab)
    lb = lab.to_array(np.int32, V).astype(np.int64)
    ok_cc = bool(np.all(lb[src] == lb[nl])) and bool(np.all(lb <= np.arange(V))) and bool(np.all(lb[lb] == lb))
    G.mis(st)
    ms = st.to_array(np.int32, V)
    x = np.arange(V, dtype=np.uint64) + np.uint64(712313887)
    x &= np.uint64(0xFFFFFFFF)
    for _ in range(2):
        x = (((x >> np.uint64(16)) ^ x) * np.uint64(0x45D9F3B)) & np.uint64(0xFFFFFFFF)
    pr = ((x >> np.uint64(16)) ^ x).astype(np.int64)
    inset = ms == 1
    larger = (pr[nl] > pr[src]) | ((pr[nl] == pr[src]) & (nl > src))  # (priority, id) order
    blocked = np.zeros(V, bool)
    blocked[src[larger & inset[nl]]] = True  # has a larger neighbour in the set
    ok_mis = bool(np.all(np.isin(ms, [1, 2]))) and bool(np.all(inset == ~blocked))
    sc = scores.to_array(np.float32, V)
    ok_pr = bool(np.all(np.isfinite(sc))) and 0.5 < float(sc.sum()) <= 1.0 + 1e-4
    GT.tc(count)
    tc = int(count.to_array(np.uint64, 1)[0])
    G.synchronize()
    return {"bfs_levels_consistent": ok_bfs, "sssp_triangle_and_tight": ok_sssp, "cc_min_label": ok_cc,
            "mis_greedy_unique": ok_mis, "pr_mass": ok_pr, "tc_count": tc}


# ----------------------------------------------------------------------------- peaks / traffic
def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        m = json.loads(p.read_text())
        return {"hbm_gbs": float(m["hbm_gbs"]), "source": "measured (MEASURED_PEAKS.json hbm_gbs, STREAM copy)"}
    return {"hbm_gbs": 6800.0, "source": "fallback 6.8 TB/s"}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per call of each
# algorithm's kernels on this workload: one ncu capture per algorithm on the
# RMAT scale-21 case (`bench.py --case <algo> --scale 21`: 63,539,260 edges),
# scaled to RMAT-22 by the edge ratio 2.019 (the traffic grows with the edges
# processed).  Kernels: sssp_persistent, pr_persistent (15 iterations),
# tc_count_block and tc_count_warp (the orientation kernels are not
# included), bfs_persistent, mis_persistent, and every kernel of the CC call
# (its seed, its BFS and the union-find kernels).  The capture and its
# figures are in the per-kernel traffic summary under profiles/.
DRAM_BYTES_PER_CALL = {"sssp": 2293121924, "pr": 8985803654, "tc": 4045317244, "bfs": 154965131,
                       "mis": 179344572, "cc": 228995045}


# ----------------------------------------------------------------------------- CPU
class CpuArm:
    """The step on this host's cores, for the reference arm and the CPU
    baseline.  kind "reference": the reference's own best-published C++
    variants (oracle/_ref/time_<algo>, compiled with g++ -O3 -pthread from its
    staged sources, scripts/run_codes.py:105), one program per algorithm
    holding its graph, each run timed by the variant's own timer; kind
    "port": the oracle's threaded restatement of the same variants
    (oracle/indigo_oracle.c) where those programs are not built.  Both use
    all host threads.  The reference's PageRank stops at its own
    EPSILON = 1e-4 (include/pr_cpp.h:45, a compile-time constant), so it does
    fewer iterations than the GPU's 1e-6; the port runs to 1e-6."""

    def __init__(self, g, gd, sources, threads: int):
        from oracle import oracle as orc
        self.orc, self.g, self.gd, self.sources, self.threads = orc, g, gd, [int(s) for s in sources], threads
        self.kind = "reference" if orc.ref_available() else "port"
        self.timers = {}
        self.tmp = None
        if self.kind == "reference":
            self.tmp = tempfile.mkdtemp(prefix="indigo_cpu_")
            egr, egr_d = os.path.join(self.tmp, "g.egr"), os.path.join(self.tmp, "gd.egr")
            g.write_egr(egr)
            gd.write_egr(egr_d)
            for a in ALGOS:
                self.timers[a] = orc.RefTimer(a, egr_d if a == "tc" else egr, threads)
            for path in (egr, egr_d):
                os.unlink(path)  # the programs hold their graphs
        self.checks = {}

    def step(self) -> tuple:
        """One full step (16 BFS + 16 SSSP + CC + MIS + PR + TC): returns the
        host wall time of the step and the per-algorithm seconds."""
        sec = {a: 0.0 for a in ALGOS}
        w0 = time.perf_counter()
        if self.kind == "reference":
            T = self.timers
            for a in ("bfs", "sssp"):
                for s in self.sources:
                    t, c = T[a].run(s)
                    sec[a] += t
                    self.checks.setdefault(a, []).append(c)
            for a in ("cc", "mis", "pr", "tc"):
                t, c = T[a].run(0)
                sec[a] += t
                self.checks[a] = c
        else:
            orc, g, T = self.orc, self.g, self.threads
            for s in self.sources:
                sec["bfs"] += orc.bfs_threads(g, s, T)[1]
            for s in self.sources:
                sec["sssp"] += orc.sssp_threads(g, s, T)[1]
            sec["cc"] = orc.cc_threads(g, T)[1]
            sec["mis"] = orc.mis_threads(g, T)[1]
            _, it, sec["pr"] = orc.pr_threads(g, T, PR_EPS, PR_MAX_ITER)
            self.checks["tc"], sec["tc"] = orc.tc_threads(self.gd, T)
        return time.perf_counter() - w0, sec

    def describe(self) -> str:
        if self.kind == "reference":
            return ("the reference's best-published C++ variants (BFS/SSSP/CC/MIS *_CPP_V_Topo_Push_*, "
                    "TC_CPP_V_IntType_Critical_Cyclic, PR_CPP_Pull_FloatType_AtomicAdd_Block_Determin) built from its "
                    "own sources with g++ -O3 -pthread, %d threads; PageRank to the reference's EPSILON 1e-4" %
                    self.threads)
        return ("the oracle's threaded restatement of the reference's best-published C++ variants "
                "(oracle/indigo_oracle.c), %d threads; the reference's programs are not built here" % self.threads)

    def close(self):
        for t in self.timers.values():
            t.close()
        if self.tmp:
            os.rmdir(self.tmp)
            self.tmp = None


def cpu_baseline(g, gd, sources, validation):
    """One full step of the workload on the host cores (no scaling): the
    value is the step's 36 runs x E over its measured wall time."""
    threads = os.cpu_count() or 1
    arm = CpuArm(g, gd, sources, threads)
    try:
        wall, sec = arm.step()
    finally:
        arm.close()
    if "tc" in arm.checks:
        validation["tc_matches_cpu"] = int(arm.checks["tc"]) == int(validation.get("tc_count", -1))
    value = RUNS_PER_STEP * g.edges / wall / 1e9
    return {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": arm.kind,
            "sample": "one full step (BFS and SSSP from all 16 sources, CC, MIS, PR, TC on the degree-ordered "
                      "graph), measured whole: %s; %.1f s wall" % (arm.describe(), wall),
            "seconds": {k: round(v, 4) for k, v in sec.items()}}


def pagerank_error(g, scores: np.ndarray, iters: int) -> dict:
    """Error of the GPU's FP32 PageRank (the bench's last call) against the
    FP64 oracle: run for the same iteration count (arithmetic error) and run
    to an L1 residual below 1e-12 (total error, including the truncation of
    stopping at the residual PR_EPS).  Relative L1 = sum|x - ref| / sum(ref);
    max = max|x - ref| / max(ref)."""
    from oracle import oracle as orc
    s64 = scores.astype(np.float64)
    same, _, _ = orc.pr_f64_threads(g, iters=iters)
    conv, it_conv, res = orc.pr_f64_threads(g)
    return {"rel_l1_vs_fp64_same_iterations": float("%.3e" % (np.abs(s64 - same).sum() / same.sum())),
            "max_rel_vs_fp64_same_iterations": float("%.3e" % (np.abs(s64 - same).max() / same.max())),
            "rel_l1_vs_fp64_converged": float("%.3e" % (np.abs(s64 - conv).sum() / conv.sum())),
            "max_rel_vs_fp64_converged": float("%.3e" % (np.abs(s64 - conv).max() / conv.max())),
            "fp64_converged_iterations": int(it_conv), "fp64_converged_residual": float("%.2e" % res)}


def run_reference(args, dist: Dist):
    """The CPU implementation on the host cores, on the same workload and
    metric.  Loads no GPU library: the graph comes from the oracle's copy of
    the generator (oracle/workload.c, proven identical by
    tests/test_oracle_workload.py).  Every step is the full workload, timed
    whole by the host clock."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    t0 = time.time()
    g = orc.gen_rmat(SCALE, EDGE_FACTOR, *RMAT_ABC, seed=SEED, maxw=MAXW, permute=True, threads=threads)
    gd = g.degree_ordered(threads)
    sources = g.pick_sources(N_SOURCES, seed=SEED)
    log(f"[bench] RMAT-{SCALE} (oracle generator): V={g.nodes} E={g.edges} in {time.time() - t0:.1f}s")
    arm = CpuArm(g, gd, sources, threads)
    try:
        for _ in range(args.warmup):
            arm.step()
        total, acc = 0.0, {a: 0.0 for a in ALGOS}
        for _ in range(args.steps):
            wall, sec = arm.step()
            total += wall
            for a in ALGOS:
                acc[a] += sec[a]
    finally:
        arm.close()
    ms_per_step = 1e3 * total / args.steps
    value = RUNS_PER_STEP * g.edges * args.steps / total / 1e9
    calls = {"bfs": N_SOURCES, "sssp": N_SOURCES, "cc": 1, "mis": 1, "pr": 1, "tc": 1}
    sample = ("every step is the full workload (BFS and SSSP from all 16 sources, CC, MIS, PR, TC on the "
              "degree-ordered graph), timed whole by the host clock: " + arm.describe())
    return {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32/f32",
            "data": "synthetic",
            "config": {"workload": f"rmat{SCALE}_ef{EDGE_FACTOR}_six_algorithms", "vertices": g.nodes,
                       "edges": g.edges, "sources": N_SOURCES, "pr_epsilon": PR_EPS},
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": arm.kind,
                             "sample": sample,
                             "seconds_per_call": {a: round(acc[a] / args.steps / calls[a], 4) for a in ALGOS}},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ----------------------------------------------------------------------------- batched form
BATCH_GRAPHS, BATCH_VMIN, BATCH_VMAX, BATCH_SEED = 4096, 1024, 65536, 13


class _At:
    """A device address with the .ptr attribute the device API takes."""

    def __init__(self, ptr: int):
        self.ptr = ptr


def run_batched(args, dist: Dist, graphs: int = BATCH_GRAPHS):
    """Configuration 4: 4096 graphs (vertex counts log-uniform in [1k, 64k],
    even Erdos-Renyi with average degree 8, odd RMAT with edge factor 8,
    weights in [1, 255], seed 13).  One step = CC, BFS from vertex 0, TC and
    PageRank of every graph with one batched call each (CUDA-graph replay);
    value = graphs/s over all ranks.  With N ranks the graphs shard with no
    exchange: "weak" gives every rank its own pack of 4096 graphs (seed 13 +
    rank), "strong" gives each rank an edge-balanced contiguous slice of the
    one pack.

    The plain comparison runs the same four algorithms on EVERY graph as one
    device-API call per graph and algorithm (each graph resident in HBM with
    its own handle, results left on the device), timed the same way as the
    batched calls: CUDA events on the one stream both use, after an untimed
    pass that sizes every handle's scratch."""
    import indigo_gb300 as ig

    ig.check(ig.load().ig_set_device(dist.local))
    t0 = time.time()
    strong = dist.world > 1 and args.batch_split == "strong"
    seed = BATCH_SEED + (0 if strong else dist.rank)
    u, vptr = ig.gen_batch(graphs, BATCH_VMIN, BATCH_VMAX, 8.0, 8, 0.57, 0.19, 0.19, seed, 255)
    if strong:
        g0, g1 = ig.split_batch(u, vptr, dist.world)[dist.rank]
        if g1 <= g0:
            raise RuntimeError(f"rank {dist.rank} received no graphs")
        u, vptr = ig.take_batch(u, vptr, g0, g1)
    graphs_here = len(vptr) - 1
    log(f"[bench] batch (rank {dist.rank}): {graphs_here} graphs, V={u.nodes} E={u.edges}, "
        f"generated in {time.time() - t0:.1f}s")
    b = ig.Batch(u, vptr)
    V = u.nodes
    d_dist, d_lab = ig.DeviceBuffer(4 * V), ig.DeviceBuffer(4 * V)
    d_cnt, d_its = ig.DeviceBuffer(8 * b.graphs), ig.DeviceBuffer(4 * b.graphs)
    sizes = np.diff(vptr)
    init = np.repeat((np.float32(1.0) / sizes.astype(np.float32)).astype(np.float32), sizes)
    d_init = ig.DeviceBuffer.from_array(init)
    d_sc = ig.DeviceBuffer(4 * V)
    L = ig.load()
    ev = {k: (ig.Event(), ig.Event()) for k in ("bfs", "cc", "tc", "pr")}
    acc = {k: 0.0 for k in ev}

    def step(timed):
        ev["cc"][0].record(b.stream)
        b.cc(d_lab)
        ev["cc"][1].record(b.stream)
        ev["bfs"][0].record(b.stream)
        b.bfs(d_dist)
        ev["bfs"][1].record(b.stream)
        ev["tc"][0].record(b.stream)
        b.tc(d_cnt)
        ev["tc"][1].record(b.stream)
        ev["pr"][0].record(b.stream)
        ig.check(L.ig_memcpy_async(d_sc.ptr, d_init.ptr, 4 * V, 3, b.stream))
        b.pagerank(d_sc, PR_EPS, PR_MAX_ITER, d_its)
        ev["pr"][1].record(b.stream)
        if timed:
            for k in ev:
                acc[k] += ev[k][0].elapsed_ms(ev[k][1])

    tuned = None
    if not args.no_autotune:
        t1 = time.time()
        tune_ms = b.autotune(("bfs", "cc", "pr"), reps=2)
        tuned = {a: {"ms": round(tune_ms[a], 3), "options": {k: b.get_option(a, k) for k in ig.Batch.TUNED[a]}}
                 for a in tune_ms}
        log(f"[bench] autotuned in {time.time() - t1:.1f}s: {tuned}")
    for _ in range(args.warmup):
        step(False)
    if b.last_run().status:
        raise RuntimeError("batched run failed")
    t_a, t_b = ig.Event(), ig.Event()
    launches0 = ig.kernel_launches()
    clocks = ClockSampler(dist.local)
    dist.barrier()
    b.synchronize()
    t_a.record(b.stream)
    for _ in range(args.steps):
        step(True)
    t_b.record(b.stream)
    b.synchronize()
    dist.barrier()
    clk = clocks.stop()
    launches = ig.kernel_launches() - launches0
    if b.last_run().status:
        raise RuntimeError("batched run failed during timing")
    its = d_its.to_array(np.int32, graphs_here)
    pr_its = {"min": int(its.min()), "median": float(np.median(its)), "max": int(its.max())}
    batch_tc = d_cnt.to_array(np.uint64, graphs_here)
    ms = dist.max(t_a.elapsed_ms(t_b)) / args.steps
    graphs_all = int(dist.sum(graphs_here))
    value = graphs_all / (ms * 1e-3)

    # plain: one device-API call per graph and algorithm, every graph
    t1 = time.time()
    handles, csrs = [], []
    for i in range(graphs_here):
        dg = ig.DeviceCSR(ig.unpack(u, vptr, i))
        G = ig.DeviceGraph(dg)
        G.set_stream(b.stream)
        csrs.append(dg)
        handles.append(G)
    vmax = int(sizes.max())
    p_dist, p_lab, p_sc = ig.DeviceBuffer(4 * vmax), ig.DeviceBuffer(4 * vmax), ig.DeviceBuffer(4 * vmax)
    p_cnt = ig.DeviceBuffer(8 * graphs_here)

    def plain_pass():
        for i, G in enumerate(handles):
            G.cc(p_lab)
            G.bfs(0, p_dist)
            G.tc(_At(p_cnt.ptr + 8 * i))
            ig.check(L.ig_memcpy_async(p_sc.ptr, d_init.ptr + 4 * int(vptr[i]), 4 * int(sizes[i]), 3, b.stream))
            G.pagerank(p_sc, PR_EPS, PR_MAX_ITER)

    plain_pass()  # sizes every handle's scratch
    b.synchronize()
    p_a, p_b = ig.Event(), ig.Event()
    p_a.record(b.stream)
    plain_pass()
    p_b.record(b.stream)
    b.synchronize()
    if any(G.last_run().status for G in handles):
        raise RuntimeError("plain per-graph run failed")
    plain_ms = dist.max(p_a.elapsed_ms(p_b))
    same_tc = bool(np.array_equal(p_cnt.to_array(np.uint64, graphs_here), batch_tc))
    plain_value = graphs_all / (plain_ms * 1e-3)
    log(f"[bench] plain per-graph pass: {plain_ms:.1f} ms ({time.time() - t1:.1f}s with uploads)")
    for G in handles:
        G.close()
    for dg in csrs:
        dg.close()
    b.close()
    return {"metric": "graphs/s (4096 packed graphs: CC + BFS + TC + PR per graph)", "value": round(value, 1),
            "unit": "graphs/s", "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "strong" if strong else "weak",
            "vs_baseline": None, "dtype": "int32/f32", "data": "synthetic",
            "config": {"workload": f"batch{graphs}_er8_rmat8", "graphs": graphs_all, "graphs_per_rank": graphs_here,
                       "vertices": V, "edges": u.edges,
                       "parallelism": (f"{dist.world} ranks, " + ("edge-balanced slices of one pack" if strong
                                       else "one pack per rank")) if dist.world > 1 else "single GPU",
                       "vmin": BATCH_VMIN, "vmax": BATCH_VMAX, "seed": BATCH_SEED,
                       "l2": "inputs larger than L2 (%.0f MB neighbour lists)" % (4 * u.edges / 1e6)},
            "per_algo_ms": {k: round(v / args.steps, 3) for k, v in acc.items()},
            "pr_iterations_per_graph": pr_its,
            "autotuned": tuned,
            "plain": {"value": round(plain_value, 1), "unit": "graphs/s", "graphs": graphs_here,
                      "ms": round(plain_ms, 3), "tc_counts_equal_batched": same_tc,
                      "api": "device API (ig_cc, ig_bfs, ig_tc, ig_pagerank), one call per graph and algorithm on "
                             "every graph, results on the device, CUDA events on the same stream"},
            "speedup_vs_plain": round(value / plain_value, 1), "clocks": clk, "gpu_launches": launches}


# ----------------------------------------------------------------------------- served form
SERVE_SCALE, SERVE_SEED = 24, 17
# offered rates (queries/s) per kind: below saturation, then the lowest rate
# of the configuration's 1k-100k sweep, which saturates both engines (every
# higher rate only lengthens the queue)
SERVE_RATES = {"bfs": [50, 100, 200, 1000], "sssp": [10, 20, 40, 1000]}
SERVE_CAP = {"bfs": 600, "sssp": 300}


def run_served(args, dist: Dist):
    """Configuration 5: resident RMAT-24 (seed 17, weights [1, 1000]); Poisson
    arrivals of single-source BFS and SSSP queries (sources uniform over
    vertices with degree > 0, 4 random targets each) at each offered rate for
    about --serve-seconds; a query's latency runs from its submission to its
    answer on the host.  Below saturation p50/p99 are service latency; at
    1000/s they include the queue.  The plain comparison answers queries one
    at a time with the drop-in calls (distances copied to the host and
    summarised there), timed the same way, from call to summary."""
    import threading

    import indigo_gb300 as ig

    ig.check(ig.load().ig_set_device(dist.local))
    t0 = time.time()
    g = ig.rmat(args.serve_scale, 16, 0.57, 0.19, 0.19, seed=SERVE_SEED, maxw=1000)
    log(f"[bench] served graph RMAT-{args.serve_scale}: V={g.nodes} E={g.edges} in {time.time() - t0:.1f}s")
    d = ig.DeviceCSR(g)
    rng = np.random.default_rng(SERVE_SEED + dist.rank)
    pool = g.pick_sources(4096, seed=SERVE_SEED)
    srv = ig.Server(d, max_pending=1 << 16)
    for k in (0, 1):  # warm-up: one of each
        srv.wait(srv.submit(k, int(pool[0])), 600000)
    per_kind = {}
    clocks = ClockSampler(dist.local)
    for kind, name in ((0, "bfs"), (1, "sssp")):
        rows = []
        for rate in SERVE_RATES[name]:
            n = int(min(SERVE_CAP[name], max(30, rate * args.serve_seconds)))
            gaps = rng.exponential(1.0 / rate, n)
            srcs = rng.choice(pool, n)
            tgts = rng.integers(0, g.nodes, (n, 4))
            tickets = [None] * n
            rejected = [0]

            def client():
                t_next = time.perf_counter()
                for i in range(n):
                    t_next += gaps[i]
                    while True:
                        now = time.perf_counter()
                        if now >= t_next:
                            break
                        if t_next - now > 2e-4:
                            time.sleep(t_next - now - 1e-4)
                    t = srv.try_submit(kind, int(srcs[i]), tgts[i])
                    if t is None:
                        rejected[0] += 1
                    tickets[i] = t

            th = threading.Thread(target=client)
            w0 = time.perf_counter()
            th.start()
            th.join()
            lat = [srv.wait(t, 600000).latency_s for t in tickets if t is not None]
            wall = time.perf_counter() - w0
            lat = np.array(lat) if lat else np.array([float("nan")])
            rows.append({"offered_qps": rate, "queries": n, "rejected": rejected[0],
                         "achieved_qps": round(len(lat) / wall, 1),
                         "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 3),
                         "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 3),
                         "saturated": bool(len(lat) / wall < 0.9 * rate)})
            log(f"[bench] served {name} @ {rate}/s: {rows[-1]}")
        # plain: one drop-in call per query, one after another
        m = args.plain_queries
        out = np.empty(g.nodes, np.int32)
        fn = ig.GPUbfs_vertex if kind == 0 else ig.GPUsssp_vertex
        fn(int(pool[1]), d, out)
        ptimes = []
        for i in range(m):
            t1 = time.perf_counter()
            fn(int(pool[2 + i]), d, out)
            ig.summarize(kind, int(pool[2 + i]), out, [0, 1, 2, 3])
            ptimes.append(time.perf_counter() - t1)
        ptimes = np.array(ptimes)
        sat = rows[-1]
        below = [r for r in rows if not r["saturated"]]
        per_kind[name] = {"rates": rows, "saturation_qps": sat["achieved_qps"],
                          "p99_ms_below_saturation": max((r["p99_ms"] for r in below), default=None),
                          "plain_qps": round(1.0 / float(ptimes.mean()), 1),
                          "plain_p50_ms": round(1e3 * float(np.percentile(ptimes, 50)), 3),
                          "plain_p99_ms": round(1e3 * float(np.percentile(ptimes, 99)), 3),
                          "speedup_vs_plain": round(sat["achieved_qps"] * float(ptimes.mean()), 1)}
    clk = clocks.stop()
    srv.close()
    d.close()
    value = dist.sum(sum(v["saturation_qps"] for v in per_kind.values()))  # one replica per rank
    return {"metric": f"served queries/s (RMAT-{args.serve_scale}, BFS and SSSP, Poisson arrivals) with p50/p99 latency",
            "value": round(value, 1), "unit": "queries/s", "n_gpus": dist.world,
            "steps": sum(len(v) for v in SERVE_RATES.values()), "warmup": 1, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": f"served_rmat{args.serve_scale}", "vertices": g.nodes, "edges": g.edges,
                       "lanes_per_engine": 64, "rates": SERVE_RATES, "targets_per_query": 4,
                       "seconds_per_rate": args.serve_seconds, "l2": "resident graph larger than L2"},
            "per_kind": per_kind, "clocks": clk}


# ----------------------------------------------------------------------------- profiling case
def run_case(args):
    """One algorithm on one synthetic graph, run --repeat times through the
    device-resident API: the small, self-contained workload that Nsight
    Compute captures use (RMAT scale 21 by default: 2,097,152 vertices, about
    63M directed edges, so the 250 MB neighbour list exceeds the 129 MB L2).
    Prints one line per run with the CUDA-event time and the algorithmic
    bytes, so that a capture can be related to the bench's roofline figures.

        python bench.py --case sssp [--scale 21 | --graph road:4096] [--repeat 1] [--opt sssp_delta=100]"""
    import indigo_gb300 as ig
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
            g = ig.rmat(int(arg), 16, seed=7, maxw=1000, permute=True)
    else:
        g = ig.rmat(args.scale, 16, seed=7, maxw=1000, permute=True)
    algo = args.case
    if algo == "tc":
        g = g.degree_ordered()
    V, E = g.nodes, g.edges
    src = int(g.pick_sources(1, seed=7)[0])
    bytes_per = {"bfs": 4 * (V + 1) + 8 * E + 4 * V, "sssp": 12 * E + 8 * V, "cc": 8 * E + 8 * V,
                 "mis": 8 * E + 12 * V, "pr": 8 * E + 20 * V, "tc": 8 * E + 4 * V}
    with ig.DeviceCSR(g) as d:
        G = ig.DeviceGraph(d)
        out = ig.DeviceBuffer(4 * V)
        cnt = ig.DeviceBuffer(8)
        init = ig.DeviceBuffer.from_array(np.full(V, np.float32(1.0) / np.float32(V), np.float32))
        a, b = ig.Event(), ig.Event()
        for r in range(args.repeat):
            if algo == "pr":
                ig.check(ig.load().ig_memcpy(out.ptr, init.ptr, 4 * V, 3))
            a.record(G.stream)
            {"bfs": lambda: G.bfs(src, out), "sssp": lambda: G.sssp(src, out), "cc": lambda: G.cc(out),
             "mis": lambda: G.mis(out), "pr": lambda: G.pagerank(out, PR_EPS, PR_MAX_ITER),
             "tc": lambda: G.tc(cnt)}[algo]()
            b.record(G.stream)
            ms = a.elapsed_ms(b)
            info = G.last_run()
            ig.check(info.status)
            mult = max(1, info.iterations) if algo == "pr" else 1
            gbs = bytes_per[algo] * mult / (ms * 1e-3) / 1e9
            print(f"{algo} run {r}: {ms:.3f} ms, iterations {info.iterations}, work {info.work}, "
                  f"aux {list(info.aux)}, {E / (ms * 1e-3) / 1e9:.2f} GTEPS, {gbs:.0f} GB/s algorithmic "
                  f"(V={V}, E={E})", flush=True)
        G.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", choices=["plain", "batched", "served"], default="plain",
                    help="plain: the six algorithms on RMAT-22 (default); batched: 4096 packed graphs; "
                         "served: queries against resident RMAT-24")
    ap.add_argument("--serve-scale", type=int, default=SERVE_SCALE)
    ap.add_argument("--no-autotune", action="store_true", help="batched form: keep the process-wide options")
    ap.add_argument("--batch-split", choices=["weak", "strong"], default="weak",
                    help="batched form with N ranks: a pack per rank (weak) or slices of one pack (strong)")
    ap.add_argument("--serve-seconds", type=float, default=3.0, help="offered-load duration per rate")
    ap.add_argument("--no-forms", action="store_true",
                    help="plain form: leave out the batched and served summaries of the default line")
    ap.add_argument("--plain-queries", type=int, default=16)
    ap.add_argument("--case", choices=ALGOS, default=None,
                    help="profiling case: run one algorithm --repeat times on --scale/--graph and print each run")
    ap.add_argument("--scale", type=int, default=21, help="profiling case: RMAT scale")
    ap.add_argument("--graph", default="", help="profiling case: rmat:<scale> | road:<side> | grid:<side>")
    ap.add_argument("--repeat", type=int, default=3, help="profiling case: runs")
    ap.add_argument("--opt", action="append", default=[], help="profiling case: kernel option name=value")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    if args.warmup < 3:
        log("[bench] warm-up raised to 3 (minimum)")
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            if dist.rank != 0:
                return
            out = run_reference(args, dist)
        elif args.form == "batched":
            out = run_batched(args, dist)
        elif args.form == "served":
            out = run_served(args, dist)
        else:
            out = run_ours(args, dist)
        if dist.rank == 0:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
