"""Batched form: many graphs packed as one disjoint union with global vertex
ids plus graph_vptr (first vertex of each graph), processed by one launch
sequence per algorithm (ig_batch_*), captured into a CUDA graph after its
first call."""
from __future__ import annotations

import ctypes
import json
import math
import os

import numpy as np

from ._lib import CSR, RunInfo, check, load
from .graph import DeviceBuffer, DeviceCSR, Graph, _take_csr


def pack(graphs: list) -> tuple:
    """Disjoint union of host graphs -> (union Graph, vptr int32[len+1])."""
    vptr = np.zeros(len(graphs) + 1, np.int64)
    eptr = np.zeros(len(graphs) + 1, np.int64)
    for i, g in enumerate(graphs):
        vptr[i + 1] = vptr[i] + g.nodes
        eptr[i + 1] = eptr[i] + g.edges
    if vptr[-1] > 2**31 - 1 or eptr[-1] > 2**31 - 1:
        raise ValueError("batch exceeds int32 vertex or edge ids")
    nindex = np.concatenate([g.nindex[:-1].astype(np.int64) + eptr[i] for i, g in enumerate(graphs)] +
                            [np.array([eptr[-1]])]).astype(np.int32)
    nlist = np.concatenate([g.nlist.astype(np.int64) + vptr[i] for i, g in enumerate(graphs)]).astype(np.int32) \
        if eptr[-1] else np.zeros(0, np.int32)
    ew = None
    if all(g.eweight is not None for g in graphs):
        ew = np.concatenate([g.eweight for g in graphs]).astype(np.int32) if eptr[-1] else np.zeros(0, np.int32)
    return Graph(nindex, nlist, ew), vptr.astype(np.int32)


def unpack(union: Graph, vptr: np.ndarray, i: int) -> Graph:
    """Graph i of a packed union, with local ids."""
    v0, v1 = int(vptr[i]), int(vptr[i + 1])
    e0, e1 = int(union.nindex[v0]), int(union.nindex[v1])
    nindex = union.nindex[v0:v1 + 1] - e0
    nlist = union.nlist[e0:e1] - v0
    ew = union.eweight[e0:e1] if union.eweight is not None else None
    return Graph(nindex, nlist, ew)


def split(union: Graph, vptr: np.ndarray, parts: int) -> list:
    """Contiguous ranges of graphs, one per part, with about equal edge
    counts (vertices break ties for edgeless packs): [(g0, g1), ...].  Used to
    spread one pack over several GPUs; graphs are independent, so no exchange
    between the parts is needed.  Part k starts at the first graph whose
    cumulative work reaches k/parts of the total."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    vptr = np.asarray(vptr, dtype=np.int64)
    graphs = len(vptr) - 1
    eptr = union.nindex.astype(np.int64)[vptr]
    work = (eptr[1:] - eptr[:-1]) + (vptr[1:] - vptr[:-1])  # edges + vertices per graph
    cum = np.concatenate([[0], np.cumsum(work)])
    total = int(cum[-1])
    bounds = [0]
    for k in range(1, parts):
        b = int(np.searchsorted(cum, total * k / parts, side="left"))
        bounds.append(min(max(b, bounds[-1]), graphs))
    bounds.append(graphs)
    return [(bounds[k], bounds[k + 1]) for k in range(parts)]


def take(union: Graph, vptr: np.ndarray, g0: int, g1: int) -> tuple:
    """Graphs [g0, g1) of a packed union as their own union (ids re-based)."""
    vptr = np.asarray(vptr, dtype=np.int64)
    v0, v1 = int(vptr[g0]), int(vptr[g1])
    e0, e1 = int(union.nindex[v0]), int(union.nindex[v1])
    nindex = (union.nindex[v0:v1 + 1].astype(np.int64) - e0).astype(np.int32)
    nlist = (union.nlist[e0:e1].astype(np.int64) - v0).astype(np.int32)
    ew = union.eweight[e0:e1].copy() if union.eweight is not None else None
    return Graph(nindex, nlist, ew), (vptr[g0:g1 + 1] - v0).astype(np.int32)


def gen_batch(graphs: int, vmin: int = 1024, vmax: int = 65536, er_degree: float = 8.0, rmat_edge_factor: int = 8,
              a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 13, maxw: int = 255) -> tuple:
    """Host generator of a batch (even: Erdos-Renyi, odd: RMAT) -> (union, vptr)."""
    out = CSR()
    vptr = np.empty(graphs + 1, np.int32)
    check(load().ig_gen_batch(graphs, vmin, vmax, er_degree, rmat_edge_factor, a, b, c, seed, maxw,
                              ctypes.byref(out), vptr.ctypes.data_as(ctypes.c_void_p)))
    return _take_csr(out), vptr


class Batch:
    def __init__(self, union: Graph, vptr: np.ndarray):
        self.union = union
        self.vptr = np.ascontiguousarray(vptr, dtype=np.int32)
        self.graphs = len(self.vptr) - 1
        self.nodes = union.nodes
        self.d = DeviceCSR(union)
        self.d_vptr = DeviceBuffer.from_array(self.vptr)
        h = ctypes.c_void_p()
        check(load().ig_batch_create(ctypes.byref(self.d.c), self.d_vptr.ptr, self.graphs, ctypes.byref(h)))
        self.h = h.value
        s = ctypes.c_void_p()
        check(load().ig_batch_stream(self.h, ctypes.byref(s)))
        self.stream = s.value

    def use_graphs(self, enable: bool):
        check(load().ig_batch_use_graphs(self.h, 1 if enable else 0))

    def bfs(self, dist: DeviceBuffer, sources: DeviceBuffer | None = None):
        check(load().ig_batch_bfs(self.h, sources.ptr if sources is not None else None, dist.ptr))

    def cc(self, label: DeviceBuffer):
        check(load().ig_batch_cc(self.h, label.ptr))

    def tc(self, counts: DeviceBuffer):
        check(load().ig_batch_tc(self.h, counts.ptr))

    def pagerank(self, scores: DeviceBuffer, epsilon: float, max_iter: int, iters: DeviceBuffer):
        check(load().ig_batch_pagerank(self.h, scores.ptr, epsilon, max_iter, iters.ptr))

    ALGOS = ("bfs", "cc", "tc", "pr")
    # the options the autotuner chooses, per algorithm (the style axes and knobs it varies)
    TUNED = {"bfs": ("blocks_per_sm", "hub_degree", "bfs_alpha", "bfs_bitmap"),
             "cc": ("hub_degree", "cc_rounds"),
             "tc": (),
             "pr": ("pr_blocks_per_sm", "pr_hub_degree", "pr_subwarp", "pr_prefetch")}

    def stats_key(self) -> str:
        """The tuning database's key for this batch: log2 buckets of the graph
        count, the mean vertex count and the mean degree."""
        v = self.nodes / max(1, self.graphs)
        deg = self.union.edges / max(1, self.nodes)
        return "g%d_v%d_d%d" % (round(math.log2(max(1, self.graphs))), round(math.log2(max(1.0, v))),
                                round(math.log2(max(1.0, deg))))

    def autotune(self, algos=("bfs", "cc", "pr"), reps: int = 2, db: str | None = None) -> dict:
        """Times the variants of each algorithm on this batch and keeps the
        fastest for later calls; returns {algo: best ms}.  With `db` (a JSON
        file path), a batch whose statistics key is stored there takes the
        stored options without timing (then ms is None), and a newly tuned
        choice is stored under its key."""
        table = {}
        if db and os.path.exists(db):
            with open(db) as f:
                table = json.load(f)
        key = self.stats_key()
        stored = table.get(key, {})
        out = {}
        todo = []
        for a in algos:
            if a in stored:
                for name, value in stored[a].items():
                    self.set_option(a, name, int(value))
                out[a] = None
            else:
                todo.append(a)
        if todo:
            mask = 0
            for a in todo:
                mask |= 1 << self.ALGOS.index(a)
            best = (ctypes.c_float * 4)()
            check(load().ig_batch_autotune(self.h, mask, reps, best))
            for a in todo:
                out[a] = float(best[self.ALGOS.index(a)])
            if db:
                entry = table.setdefault(key, {})
                for a in todo:
                    entry[a] = {n: self.get_option(a, n) for n in self.TUNED[a]}
                tmp = db + ".tmp"
                with open(tmp, "w") as f:
                    json.dump(table, f, indent=1, sort_keys=True)
                os.replace(tmp, db)
        return out

    def set_option(self, algo: str, name: str, value: int):
        check(load().ig_batch_set_option(self.h, self.ALGOS.index(algo), name.encode(), int(value)))

    def get_option(self, algo: str, name: str) -> int:
        v = ctypes.c_longlong()
        check(load().ig_batch_get_option(self.h, self.ALGOS.index(algo), name.encode(), ctypes.byref(v)))
        return v.value

    def last_run(self) -> RunInfo:
        info = RunInfo()
        check(load().ig_batch_last_run(self.h, ctypes.byref(info)))
        return info

    def synchronize(self):
        check(load().ig_stream_synchronize(self.stream))

    def close(self):
        if getattr(self, "h", None):
            load().ig_batch_destroy(self.h)
            self.h = None
            self.d.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
