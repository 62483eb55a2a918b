"""Device-resident graph API (ig_graph_*): the graph stays in HBM, results go
to device buffers, calls are asynchronous on the graph's stream."""
from __future__ import annotations

import ctypes

from ._lib import RunInfo, check, load
from .graph import DeviceBuffer, DeviceCSR


class DeviceGraph:
    def __init__(self, d: DeviceCSR):
        self.d = d
        self.nodes, self.edges = d.nodes, d.edges
        h = ctypes.c_void_p()
        check(load().ig_graph_create(ctypes.byref(d.c), ctypes.byref(h)))
        self.h = h.value
        s = ctypes.c_void_p()
        check(load().ig_graph_stream(self.h, ctypes.byref(s)))
        self.stream = s.value

    def set_stream(self, stream):
        check(load().ig_graph_set_stream(self.h, stream))
        s = ctypes.c_void_p()
        check(load().ig_graph_stream(self.h, ctypes.byref(s)))
        self.stream = s.value

    def bfs(self, src: int, dist: DeviceBuffer):
        check(load().ig_bfs(self.h, src, dist.ptr))

    def sssp(self, src: int, dist: DeviceBuffer):
        check(load().ig_sssp(self.h, src, dist.ptr))

    def cc(self, label: DeviceBuffer):
        check(load().ig_cc(self.h, label.ptr))

    def mis(self, status: DeviceBuffer):
        check(load().ig_mis(self.h, status.ptr))

    def pagerank(self, scores: DeviceBuffer, epsilon: float, max_iter: int):
        check(load().ig_pagerank(self.h, scores.ptr, epsilon, max_iter))

    def tc(self, count: DeviceBuffer):
        check(load().ig_tc(self.h, count.ptr))

    def last_run(self) -> RunInfo:
        info = RunInfo()
        check(load().ig_graph_last_run(self.h, ctypes.byref(info)))
        return info

    def synchronize(self):
        check(load().ig_stream_synchronize(self.stream))

    def close(self):
        if getattr(self, "h", None):
            load().ig_graph_destroy(self.h)
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


class Event:
    def __init__(self):
        e = ctypes.c_void_p()
        check(load().ig_event_create(ctypes.byref(e)))
        self.e = e.value

    def record(self, stream):
        check(load().ig_event_record(self.e, stream))

    def elapsed_ms(self, end: "Event") -> float:
        ms = ctypes.c_float()
        check(load().ig_event_elapsed_ms(self.e, end.e, ctypes.byref(ms)))
        return ms.value

    def __del__(self):
        try:
            load().ig_event_destroy(self.e)
        except Exception:
            pass


def set_option(name: str, value: int):
    check(load().ig_set_option(name.encode(), int(value)))


def get_option(name: str) -> int:
    v = ctypes.c_longlong()
    check(load().ig_get_option(name.encode(), ctypes.byref(v)))
    return v.value


def kernel_launches() -> int:
    n = ctypes.c_longlong()
    check(load().ig_kernel_launches(ctypes.byref(n)))
    return n.value


def create_stream():
    s = ctypes.c_void_p()
    check(load().ig_stream_create(ctypes.byref(s)))
    return s.value


def set_wait_timeout_ms(ms: int):
    check(load().ig_set_wait_timeout_ms(int(ms)))


def probe_random_gather(table_elems: int, gathers: int = 1 << 29, reps: int = 3) -> float:
    """Random 4-byte reads per second from a table of table_elems floats
    (ig_probe_random_gather): the ceiling of data-dependent graph reads."""
    out = ctypes.c_double()
    check(load().ig_probe_random_gather(table_elems, gathers, reps, ctypes.byref(out)))
    return out.value
