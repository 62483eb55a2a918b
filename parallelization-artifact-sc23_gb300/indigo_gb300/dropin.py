"""Host-side mirror of the reference's entry functions, with the same names,
argument meaning and pointer residency (include/*_cuda.h), each forwarding to
the C ABI.  Where the reference returns through a C++ reference parameter
(`basic_t& count`) the Python form returns it; the reference prints and
exits on errors, these raise IndigoError."""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import CSR, check, load
from .graph import DeviceCSR, Graph


def _out(arr: np.ndarray, n: int, dtype) -> np.ndarray:
    if arr.dtype != dtype or arr.shape[0] < n or not arr.flags.c_contiguous:
        raise ValueError(f"output must be a contiguous {np.dtype(dtype).name} array of >= {n} entries")
    return arr


def GPUbfs_vertex(src: int, d_g: DeviceCSR, dist: np.ndarray) -> float:
    """include/bfs_vertex_cuda.h:61 -- device graph, host dist[nodes]; seconds."""
    _out(dist, d_g.nodes, np.int32)
    t = ctypes.c_double()
    check(load().ig_bfs_vertex(src, ctypes.byref(d_g.c), dist.ctypes.data, ctypes.byref(t)))
    return t.value


def GPUsssp_vertex(src: int, d_g: DeviceCSR, dist: np.ndarray) -> float:
    """include/sssp_vertex_cuda.h:60."""
    _out(dist, d_g.nodes, np.int32)
    t = ctypes.c_double()
    check(load().ig_sssp_vertex(src, ctypes.byref(d_g.c), dist.ctypes.data, ctypes.byref(t)))
    return t.value


def GPUcc_vertex(d_g: DeviceCSR, label: np.ndarray) -> float:
    """include/cc_vertex_cuda.h:57."""
    _out(label, d_g.nodes, np.int32)
    t = ctypes.c_double()
    check(load().ig_cc_vertex(ctypes.byref(d_g.c), label.ctypes.data, ctypes.byref(t)))
    return t.value


def GPUmis_vertex(d_g: DeviceCSR, priority: np.ndarray | None, status: np.ndarray) -> float:
    """include/mis_vertex_cuda.h:54 -- status[v] = 1 (in) / 2 (out)."""
    _out(status, d_g.nodes, np.int32)
    pp = None
    if priority is not None:
        _out(priority, d_g.nodes, np.uint32)
        pp = priority.ctypes.data
    t = ctypes.c_double()
    check(load().ig_mis_vertex(ctypes.byref(d_g.c), pp, status.ctypes.data, ctypes.byref(t)))
    return t.value


def PR_GPU(g: Graph, scores: np.ndarray, degree: np.ndarray, epsilon: float = 1e-4, max_iter: int = 100):
    """include/pr_cuda.h:48 -- HOST graph; scores float32 in/out.  Returns
    (iterations, seconds); the reference prints them."""
    _out(scores, g.nodes, np.float32)
    _out(degree, g.nodes, np.int32)
    c = g.csr()
    it = ctypes.c_int()
    t = ctypes.c_double()
    check(load().ig_pr(ctypes.byref(c), scores.ctypes.data, degree.ctypes.data, epsilon, max_iter,
                       ctypes.byref(it), ctypes.byref(t)))
    return it.value, t.value


def GPUtc_vertex(nodes: int, d_nindex: int, d_nlist: int):
    """include/tc_vertex_cuda.h:42 -- device nindex/nlist pointers.
    Returns (count, seconds)."""
    cnt = ctypes.c_longlong()
    t = ctypes.c_double()
    check(load().ig_tc_vertex(ctypes.byref(cnt), nodes, d_nindex, d_nlist, ctypes.byref(t)))
    return int(cnt.value), t.value


# ---------------------------------------------------------------- edge forms
def GPUbfs_edge(src: int, d_g: DeviceCSR, dist: np.ndarray, sp: np.ndarray) -> float:
    """include/bfs_edge_cuda.h:61 -- sp: host COO source array."""
    _out(dist, d_g.nodes, np.int32)
    sp = np.ascontiguousarray(sp, dtype=np.int32)
    t = ctypes.c_double()
    check(load().ig_bfs_edge(src, ctypes.byref(d_g.c), dist.ctypes.data, sp.ctypes.data, ctypes.byref(t)))
    return t.value


def GPUsssp_edge(src: int, d_g: DeviceCSR, dist: np.ndarray, sp: np.ndarray) -> float:
    """include/sssp_edge_cuda.h:60."""
    _out(dist, d_g.nodes, np.int32)
    sp = np.ascontiguousarray(sp, dtype=np.int32)
    t = ctypes.c_double()
    check(load().ig_sssp_edge(src, ctypes.byref(d_g.c), dist.ctypes.data, sp.ctypes.data, ctypes.byref(t)))
    return t.value


def GPUcc_edge(d_g: DeviceCSR, label: np.ndarray, sp: np.ndarray) -> float:
    """include/cc_edge_cuda.h:57."""
    _out(label, d_g.nodes, np.int32)
    sp = np.ascontiguousarray(sp, dtype=np.int32)
    t = ctypes.c_double()
    check(load().ig_cc_edge(ctypes.byref(d_g.c), label.ctypes.data, sp.ctypes.data, ctypes.byref(t)))
    return t.value


def GPUmis_edge(d_g: DeviceCSR, d_sp: int, priority: np.ndarray | None, status: np.ndarray) -> float:
    """include/mis_edge_cuda.h:54 -- d_sp: DEVICE COO source array (the driver
    uploads it, include/mis_edge_cuda.h:154-161); status[v] = 1 (in) / 2 (out)."""
    _out(status, d_g.nodes, np.int32)
    pp = None
    if priority is not None:
        _out(priority, d_g.nodes, np.uint32)
        pp = priority.ctypes.data
    t = ctypes.c_double()
    check(load().ig_mis_edge(ctypes.byref(d_g.c), d_sp, pp, status.ctypes.data, ctypes.byref(t)))
    return t.value


def GPUtc_edge(edges: int, d_nindex: int, d_nlist: int, d_sp: int):
    """include/tc_edge_cuda.h:42 -- device nindex/nlist/sp pointers.
    Returns (count, seconds)."""
    cnt = ctypes.c_longlong()
    t = ctypes.c_double()
    check(load().ig_tc_edge(ctypes.byref(cnt), edges, d_nindex, d_nlist, d_sp, ctypes.byref(t)))
    return int(cnt.value), t.value
