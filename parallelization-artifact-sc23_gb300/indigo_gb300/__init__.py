"""GB300 (sm_103a) implementation of the Indigo2 graph-analytics hot path:
BFS, SSSP, CC, MIS, PageRank and triangle counting over ECLgraph CSR.

The compute runs in libindigo_gb300.so (hand-written CUDA kernels behind a C
ABI, include/indigo_gb300.h); this package is the Python host-side mirror of
the reference entry functions plus the device-resident graph API."""
from ._lib import CSR, IndigoError, RunInfo, check, load, LIB_PATH  # noqa: F401
from .graph import (DeviceBuffer, DeviceCSR, Graph, device_count, erdos_renyi, grid2d,  # noqa: F401
                    read_egr, rmat, road)
from .dropin import (GPUbfs_edge, GPUbfs_vertex, GPUcc_edge, GPUcc_vertex, GPUmis_edge, GPUmis_vertex,  # noqa: F401
                     GPUsssp_edge, GPUsssp_vertex, GPUtc_edge, GPUtc_vertex, PR_GPU)
from .device import (DeviceGraph, Event, create_stream, get_option, kernel_launches, probe_random_gather,  # noqa: F401
                     set_option,  # noqa: F401
                     set_wait_timeout_ms)

from .batch import Batch, gen_batch, pack, unpack  # noqa: F401
from .batch import split as split_batch, take as take_batch  # noqa: F401
from .serve import Answer, Server, summarize  # noqa: F401

INT_MAX = 2147483647
