"""Served form: BFS / SSSP queries against a resident graph (ig_server_*).

A native worker thread answers queries with 64-lane multi-source traversals
and continuous batching; a query returns its summary (vertices reached,
largest and summed finite distance, distances to up to 16 targets)."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from ._lib import IG_ERR_BUSY, IndigoError, QueryResult, check, load
from .graph import DeviceCSR

BFS, SSSP = 0, 1
INT_MAX = 2147483647


@dataclass
class Answer:
    kind: int
    source: int
    reached: int
    max_dist: int
    sum_dist: int
    targets: list = field(default_factory=list)
    target_dist: list = field(default_factory=list)
    latency_s: float = 0.0
    queue_s: float = 0.0

    def key(self):
        return (self.kind, self.source, self.reached, self.max_dist, self.sum_dist, tuple(self.targets),
                tuple(self.target_dist))


def summarize(kind: int, source: int, dist: np.ndarray, targets=()) -> Answer:
    """The served answer computed from a full distance vector (for checks and
    for the plain one-call-per-query comparison)."""
    fin = dist[dist != INT_MAX].astype(np.int64)
    return Answer(kind, int(source), int(fin.size), int(fin.max()) if fin.size else 0, int(fin.sum()),
                  [int(t) for t in targets], [int(dist[t]) for t in targets])


class Server:
    def __init__(self, d: DeviceCSR, max_pending: int = 4096):
        self.d = d
        h = ctypes.c_void_p()
        check(load().ig_server_create(ctypes.byref(d.c), max_pending, ctypes.byref(h)))
        self.h = h.value

    def submit(self, kind: int, source: int, targets=()) -> int:
        t = np.ascontiguousarray(np.asarray(targets, dtype=np.int32))
        ticket = ctypes.c_longlong()
        check(load().ig_server_submit(self.h, kind, int(source), t.ctypes.data if t.size else None, int(t.size),
                                      ctypes.byref(ticket)))
        return ticket.value

    def try_submit(self, kind: int, source: int, targets=()):
        """submit() that returns None instead of raising when the queue is full."""
        try:
            return self.submit(kind, source, targets)
        except IndigoError as e:
            if e.status == IG_ERR_BUSY:
                return None
            raise

    def wait(self, ticket: int, timeout_ms: int = 60000) -> Answer:
        r = QueryResult()
        check(load().ig_server_wait(self.h, ticket, timeout_ms, ctypes.byref(r)))
        check(r.status)
        n = r.ntargets
        return Answer(r.kind, r.source, r.reached, r.max_dist, r.sum_dist, list(r.targets[:n]),
                      list(r.target_dist[:n]), r.done_time - r.submit_time, r.admit_time - r.submit_time)

    def stats(self):
        c, s = ctypes.c_longlong(), ctypes.c_longlong()
        check(load().ig_server_stats(self.h, ctypes.byref(c), ctypes.byref(s)))
        return c.value, s.value

    def set_memory_budget(self, nbytes: int):
        """Caps the device bytes the engines may hold together (-1: no cap)."""
        check(load().ig_server_set_memory_budget(self.h, int(nbytes)))

    def memory(self):
        """(bytes the engines hold, admissions deferred for memory, engines created)."""
        h, d, c = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        check(load().ig_server_memory(self.h, ctypes.byref(h), ctypes.byref(d), ctypes.byref(c)))
        return h.value, d.value, c.value

    def close(self):
        if getattr(self, "h", None):
            load().ig_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
