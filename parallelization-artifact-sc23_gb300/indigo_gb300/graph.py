"""Host and device CSR graphs over the library's C ABI.

`Graph` mirrors the reference's struct ECLgraph (include/ECLgraph.h:44-50)
with numpy arrays: nodes, edges, nindex[nodes+1], nlist[edges] and optional
eweight[edges]."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from ._lib import CSR, check, load


def _take_csr(c: CSR) -> "Graph":
    """Copies a library-allocated host CSR into numpy arrays and frees it."""
    L = load()
    try:
        n, e = c.nodes, c.edges
        nindex = np.ctypeslib.as_array(c.nindex, shape=(n + 1,)).copy()
        nlist = np.ctypeslib.as_array(c.nlist, shape=(max(e, 1),))[:e].copy() if e > 0 else np.zeros(0, np.int32)
        ew = None
        if c.eweight:
            ew = np.ctypeslib.as_array(c.eweight, shape=(max(e, 1),))[:e].copy() if e > 0 else np.zeros(0, np.int32)
        return Graph(nindex.astype(np.int32), nlist.astype(np.int32), None if ew is None else ew.astype(np.int32))
    finally:
        L.ig_csr_free_host(ctypes.byref(c))


@dataclass
class Graph:
    nindex: np.ndarray
    nlist: np.ndarray
    eweight: Optional[np.ndarray] = None

    def __post_init__(self):
        self.nindex = np.ascontiguousarray(self.nindex, dtype=np.int32)
        self.nlist = np.ascontiguousarray(self.nlist, dtype=np.int32)
        if self.eweight is not None:
            self.eweight = np.ascontiguousarray(self.eweight, dtype=np.int32)

    @property
    def nodes(self) -> int:
        return int(self.nindex.shape[0] - 1)

    @property
    def edges(self) -> int:
        return int(self.nlist.shape[0])

    def degree(self) -> np.ndarray:
        return np.diff(self.nindex).astype(np.int32)

    def csr(self) -> CSR:
        """ig_csr view of the numpy arrays (valid while this Graph lives)."""
        ip = ctypes.POINTER(ctypes.c_int)
        c = CSR()
        c.nodes, c.edges = self.nodes, self.edges
        c.nindex = self.nindex.ctypes.data_as(ip)
        c.nlist = self.nlist.ctypes.data_as(ip) if self.edges else self.nlist.ctypes.data_as(ip)
        c.eweight = self.eweight.ctypes.data_as(ip) if self.eweight is not None else ip()
        return c

    def digest(self) -> int:
        c = self.csr()
        return int(load().ig_csr_digest(ctypes.byref(c)))

    def write_egr(self, path: str) -> None:
        c = self.csr()
        check(load().ig_egr_write(str(path).encode(), ctypes.byref(c)))

    def sp(self) -> np.ndarray:
        """COO source array sp[e] (the reference edge drivers build it, e.g.
        include/sssp_edge_cuda.h:149-155)."""
        return np.repeat(np.arange(self.nodes, dtype=np.int32), self.degree())

    def degree_ordered(self) -> "Graph":
        c = self.csr()
        out = CSR()
        check(load().ig_degree_order(ctypes.byref(c), ctypes.byref(out)))
        return _take_csr(out)

    def pick_sources(self, k: int, seed: int) -> np.ndarray:
        c = self.csr()
        out = np.empty(k, dtype=np.int32)
        check(load().ig_pick_sources(ctypes.byref(c), k, seed, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def is_sorted(self) -> bool:
        c = self.csr()
        return load().ig_csr_check_sorted(ctypes.byref(c)) == 0


def read_egr(path: str) -> Graph:
    out = CSR()
    check(load().ig_egr_read(str(path).encode(), ctypes.byref(out)))
    return _take_csr(out)


def grid2d(nx: int, ny: int, maxw: int = 0, seed: int = 1) -> Graph:
    out = CSR()
    check(load().ig_gen_grid2d(nx, ny, maxw, seed, ctypes.byref(out)))
    return _take_csr(out)


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 7,
         maxw: int = 0, permute: bool = True) -> Graph:
    out = CSR()
    check(load().ig_gen_rmat(scale, edge_factor, a, b, c, seed, maxw, 1 if permute else 0, ctypes.byref(out)))
    return _take_csr(out)


def road(nx: int, ny: int, delete_frac: float = 0.05, shortcut_frac: float = 0.001, seed: int = 11,
         maxw: int = 10000) -> Graph:
    out = CSR()
    check(load().ig_gen_road(nx, ny, delete_frac, shortcut_frac, seed, maxw, ctypes.byref(out)))
    return _take_csr(out)


def erdos_renyi(n: int, avg_degree: float = 8.0, seed: int = 13, maxw: int = 0) -> Graph:
    out = CSR()
    check(load().ig_gen_er(n, avg_degree, seed, maxw, ctypes.byref(out)))
    return _take_csr(out)


class DeviceBuffer:
    """A device allocation owned by Python (freed on close/GC)."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        check(load().ig_dev_alloc(ctypes.byref(p), max(1, self.nbytes)))
        self.ptr = p.value

    @classmethod
    def from_array(cls, a: np.ndarray) -> "DeviceBuffer":
        a = np.ascontiguousarray(a)
        buf = cls(a.nbytes)
        if a.nbytes:
            check(load().ig_memcpy(buf.ptr, a.ctypes.data, a.nbytes, 1))
        return buf

    def to_array(self, dtype, count: int) -> np.ndarray:
        out = np.empty(count, dtype=dtype)
        if out.nbytes:
            check(load().ig_memcpy(out.ctypes.data, self.ptr, out.nbytes, 2))
        return out

    def close(self):
        if getattr(self, "ptr", None):
            load().ig_dev_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceCSR:
    """A graph copied to device memory (ig_csr_upload); the drop-in entry
    points take it where the reference passes its device ECLgraph d_g."""

    def __init__(self, g: Graph):
        self.host = g
        self.c = CSR()
        h = g.csr()
        check(load().ig_csr_upload(ctypes.byref(h), ctypes.byref(self.c)))
        self.nodes, self.edges = g.nodes, g.edges

    @property
    def nindex_ptr(self) -> int:
        return ctypes.cast(self.c.nindex, ctypes.c_void_p).value

    @property
    def nlist_ptr(self) -> int:
        return ctypes.cast(self.c.nlist, ctypes.c_void_p).value

    @classmethod
    def _adopt(cls, c: CSR) -> "DeviceCSR":
        """Wraps device arrays the library allocated (freed by close)."""
        d = cls.__new__(cls)
        d.host, d.c, d.nodes, d.edges = None, c, c.nodes, c.edges
        return d

    def prepare(self, symmetrize: bool = False, degree_order: bool = False) -> "DeviceCSR":
        """ig_csr_prepare: a new device graph without self loops or duplicate
        edges and with sorted lists; optionally symmetrised and relabelled in
        (degree, id) order."""
        out = CSR()
        flags = (1 if symmetrize else 0) | (2 if degree_order else 0)
        check(load().ig_csr_prepare(ctypes.byref(self.c), flags, ctypes.byref(out)))
        return DeviceCSR._adopt(out)

    def to_graph(self) -> Graph:
        """Copies the device arrays back into a host Graph."""
        L = load()
        ni = np.empty(self.nodes + 1, np.int32)
        nl = np.empty(max(1, self.edges), np.int32)
        check(L.ig_memcpy(ni.ctypes.data, ctypes.cast(self.c.nindex, ctypes.c_void_p), ni.nbytes, 2))
        check(L.ig_memcpy(nl.ctypes.data, ctypes.cast(self.c.nlist, ctypes.c_void_p), nl.nbytes, 2))
        ew = None
        if self.c.eweight:
            ew = np.empty(max(1, self.edges), np.int32)
            check(L.ig_memcpy(ew.ctypes.data, ctypes.cast(self.c.eweight, ctypes.c_void_p), ew.nbytes, 2))
            ew = ew[: self.edges]
        return Graph(ni, nl[: self.edges], ew)

    def close(self):
        if self.c.nindex:
            load().ig_csr_free_device(ctypes.byref(self.c))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_count() -> int:
    n = ctypes.c_int(0)
    st = load().ig_device_count(ctypes.byref(n))
    return n.value if st == 0 else 0
