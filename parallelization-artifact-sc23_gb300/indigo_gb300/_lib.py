"""ctypes binding of libindigo_gb300.so (the C ABI in include/indigo_gb300.h).

The shared library is built in-tree by ../build.py; importing this module
without it raises IndigoError (there is no CPU fallback)."""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libindigo_gb300.so"


class IndigoError(RuntimeError):
    """A library call returned a non-zero ig_status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


IG_OK = 0
IG_ERR_INVALID_ARG = 1
IG_ERR_CUDA = 2
IG_ERR_NOMEM = 3
IG_ERR_TIMEOUT = 4
IG_ERR_UNSORTED = 5
IG_ERR_NO_DEVICE = 6
IG_ERR_OVERFLOW = 7
IG_ERR_IO = 8
IG_ERR_FORMAT = 9
IG_ERR_BUSY = 10
IG_ERR_CANCELLED = 11


class CSR(ctypes.Structure):
    """struct ig_csr, layout-compatible with the reference's struct ECLgraph."""

    _fields_ = [
        ("nodes", ctypes.c_int),
        ("edges", ctypes.c_int),
        ("nindex", ctypes.POINTER(ctypes.c_int)),
        ("nlist", ctypes.POINTER(ctypes.c_int)),
        ("eweight", ctypes.POINTER(ctypes.c_int)),
    ]


class QueryResult(ctypes.Structure):
    """struct ig_query_result."""

    _fields_ = [
        ("status", ctypes.c_int),
        ("kind", ctypes.c_int),
        ("source", ctypes.c_int),
        ("levels", ctypes.c_int),
        ("reached", ctypes.c_longlong),
        ("max_dist", ctypes.c_longlong),
        ("sum_dist", ctypes.c_longlong),
        ("ntargets", ctypes.c_int),
        ("targets", ctypes.c_int * 16),
        ("target_dist", ctypes.c_int * 16),
        ("submit_time", ctypes.c_double),
        ("admit_time", ctypes.c_double),
        ("done_time", ctypes.c_double),
    ]


class RunInfo(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("iterations", ctypes.c_int),
        ("work", ctypes.c_longlong),
        ("residual", ctypes.c_double),
        ("aux", ctypes.c_longlong * 4),
    ]


_I = ctypes.c_int
_P = ctypes.c_void_p
_PCSR = ctypes.POINTER(CSR)
_PI = ctypes.POINTER(ctypes.c_int)
_PD = ctypes.POINTER(ctypes.c_double)
_U64 = ctypes.c_uint64

# name -> (restype, argtypes)
SIGNATURES = {
    "ig_status_string": (ctypes.c_char_p, [_I]),
    "ig_last_error": (ctypes.c_char_p, []),
    "ig_version": (_I, []),
    "ig_egr_read": (_I, [ctypes.c_char_p, _PCSR]),
    "ig_egr_write": (_I, [ctypes.c_char_p, _PCSR]),
    "ig_csr_free_host": (None, [_PCSR]),
    "ig_gen_grid2d": (_I, [_I, _I, _I, _U64, _PCSR]),
    "ig_gen_rmat": (_I, [_I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double, _U64, _I, _I, _PCSR]),
    "ig_gen_road": (_I, [_I, _I, ctypes.c_double, ctypes.c_double, _U64, _I, _PCSR]),
    "ig_gen_er": (_I, [_I, ctypes.c_double, _U64, _I, _PCSR]),
    "ig_degree_order": (_I, [_PCSR, _PCSR]),
    "ig_pick_sources": (_I, [_PCSR, _I, _U64, _P]),
    "ig_csr_check_sorted": (_I, [_PCSR]),
    "ig_csr_digest": (_U64, [_PCSR]),
    "ig_device_count": (_I, [_PI]),
    "ig_set_device": (_I, [_I]),
    "ig_device_name": (_I, [ctypes.c_char_p, _I]),
    "ig_device_memory": (_I, [ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_ulonglong)]),
    "ig_dev_alloc": (_I, [ctypes.POINTER(_P), ctypes.c_size_t]),
    "ig_dev_free": (_I, [_P]),
    "ig_host_alloc_pinned": (_I, [ctypes.POINTER(_P), ctypes.c_size_t]),
    "ig_host_free_pinned": (_I, [_P]),
    "ig_memcpy": (_I, [_P, _P, ctypes.c_size_t, _I]),
    "ig_memcpy_async": (_I, [_P, _P, ctypes.c_size_t, _I, _P]),
    "ig_memset": (_I, [_P, _I, ctypes.c_size_t]),
    "ig_device_synchronize": (_I, []),
    "ig_csr_upload": (_I, [_PCSR, _PCSR]),
    "ig_csr_free_device": (_I, [_PCSR]),
    "ig_csr_prepare": (_I, [_PCSR, _I, _PCSR]),
    "ig_stream_create": (_I, [ctypes.POINTER(_P)]),
    "ig_stream_destroy": (_I, [_P]),
    "ig_stream_create_nonblocking": (_I, [ctypes.POINTER(_P)]),
    "ig_probe_random_gather": (_I, [ctypes.c_longlong, ctypes.c_longlong, _I, ctypes.POINTER(ctypes.c_double)]),
    "ig_stream_synchronize": (_I, [_P]),
    "ig_event_create": (_I, [ctypes.POINTER(_P)]),
    "ig_event_destroy": (_I, [_P]),
    "ig_event_record": (_I, [_P, _P]),
    "ig_event_elapsed_ms": (_I, [_P, _P, ctypes.POINTER(ctypes.c_float)]),
    "ig_set_wait_timeout_ms": (_I, [_I]),
    "ig_set_option": (_I, [ctypes.c_char_p, ctypes.c_longlong]),
    "ig_get_option": (_I, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong)]),
    "ig_bfs_vertex": (_I, [_I, _PCSR, _P, _PD]),
    "ig_sssp_vertex": (_I, [_I, _PCSR, _P, _PD]),
    "ig_cc_vertex": (_I, [_PCSR, _P, _PD]),
    "ig_mis_vertex": (_I, [_PCSR, _P, _P, _PD]),
    "ig_pr": (_I, [_PCSR, _P, _P, ctypes.c_float, _I, _PI, _PD]),
    "ig_tc_vertex": (_I, [ctypes.POINTER(ctypes.c_longlong), _I, _P, _P, _PD]),
    "ig_bfs_edge": (_I, [_I, _PCSR, _P, _P, _PD]),
    "ig_sssp_edge": (_I, [_I, _PCSR, _P, _P, _PD]),
    "ig_cc_edge": (_I, [_PCSR, _P, _P, _PD]),
    "ig_mis_edge": (_I, [_PCSR, _P, _P, _P, _PD]),
    "ig_tc_edge": (_I, [ctypes.POINTER(ctypes.c_longlong), _I, _P, _P, _P, _PD]),
    "ig_graph_create": (_I, [_PCSR, ctypes.POINTER(_P)]),
    "ig_graph_destroy": (_I, [_P]),
    "ig_graph_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "ig_graph_last_run": (_I, [_P, ctypes.POINTER(RunInfo)]),
    "ig_bfs": (_I, [_P, _I, _P]),
    "ig_sssp": (_I, [_P, _I, _P]),
    "ig_cc": (_I, [_P, _P]),
    "ig_mis": (_I, [_P, _P]),
    "ig_pagerank": (_I, [_P, _P, ctypes.c_float, _I]),
    "ig_tc": (_I, [_P, _P]),
    "ig_selftest_wait_timeout": (_I, [_I, _PI]),
    "ig_graph_set_stream": (_I, [_P, _P]),
    "ig_kernel_launches": (_I, [ctypes.POINTER(ctypes.c_longlong)]),
    "ig_bfs_vertex_noalloc": (_I, [_I, _PCSR, _P, _P]),
    "ig_batch_create": (_I, [_PCSR, _P, _I, ctypes.POINTER(_P)]),
    "ig_batch_destroy": (_I, [_P]),
    "ig_batch_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "ig_batch_use_graphs": (_I, [_P, _I]),
    "ig_batch_last_run": (_I, [_P, ctypes.POINTER(RunInfo)]),
    "ig_batch_bfs": (_I, [_P, _P, _P]),
    "ig_batch_cc": (_I, [_P, _P]),
    "ig_batch_tc": (_I, [_P, _P]),
    "ig_batch_pagerank": (_I, [_P, _P, ctypes.c_float, _I, _P]),
    "ig_batch_autotune": (_I, [_P, _I, _I, _P]),
    "ig_batch_get_option": (_I, [_P, _I, ctypes.c_char_p, _P]),
    "ig_batch_set_option": (_I, [_P, _I, ctypes.c_char_p, ctypes.c_longlong]),
    "ig_server_create": (_I, [_PCSR, _I, ctypes.POINTER(_P)]),
    "ig_server_submit": (_I, [_P, _I, _I, _P, _I, ctypes.POINTER(ctypes.c_longlong)]),
    "ig_server_wait": (_I, [_P, ctypes.c_longlong, _I, ctypes.POINTER(QueryResult)]),
    "ig_server_stats": (_I, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    "ig_server_destroy": (_I, [_P]),
    "ig_server_set_memory_budget": (_I, [_P, ctypes.c_longlong]),
    "ig_server_memory": (_I, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                              ctypes.POINTER(ctypes.c_longlong)]),
    "ig_gen_batch": (_I, [_I, _I, _I, ctypes.c_double, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double, _U64,
                          _I, _PCSR, _P]),
}

_lib = None


def load():
    """Loads and types the library once; raises IndigoError when it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise IndigoError(IG_ERR_CUDA, f"{LIB_PATH} is not built; run parallelization-artifact-sc23_gb300/build.py")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != IG_OK:
        L = load()
        msg = (L.ig_last_error() or b"").decode(errors="replace") or L.ig_status_string(status).decode()
        raise IndigoError(status, msg)
