"""TEST INFRASTRUCTURE ONLY: ctypes loader for the CPU oracle
(oracle/indigo_oracle.c) and runners for the reference's own C++ programs
built into oracle/_ref/ by oracle/build_ref.sh.

The GPU library never imports this module; tests, smoke() and bench.py's
CPU-baseline leg use it as the checker / CPU baseline."""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SO = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

_I = ctypes.c_int
_P = ctypes.c_void_p


def build(force: bool = False) -> Path:
    srcs = [HERE / "indigo_oracle.c", HERE / "workload.c"]
    newest = max(s.stat().st_mtime for s in srcs)
    if force or not SO.exists() or SO.stat().st_mtime < newest:
        tmp = SO.with_suffix(".so.tmp")
        cmd = [os.environ.get("CC", "gcc"), "-O3", "-fPIC", "-shared", "-pthread", "-std=c11",
               "-ffp-contract=off", "-D_POSIX_C_SOURCE=200809L", *map(str, srcs), "-o", str(tmp), "-lm"]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        os.replace(tmp, SO)
    return SO


REF_SRC = REF_DIR / "src"
REF_PROGRAMS = [f"{k}_{a}" for k in ("ref", "time") for a in ("bfs", "sssp", "cc", "mis", "pr", "tc")]


def stage_ref() -> bool:
    """Stages the reference files the programs compile against into
    oracle/_ref/src (oracle/stage_ref.sh; a no-op where the reference tree is
    absent).  Returns whether staged sources are present."""
    subprocess.run(["sh", str(HERE / "stage_ref.sh")], check=True, capture_output=True, text=True)
    return ref_sources_present()


def ref_sources_present() -> bool:
    """Whether the reference's sources are staged here (build_ref can run)."""
    return (REF_SRC / "include" / "ECLgraph.h").is_file()


def build_ref() -> bool:
    """Stages (where the reference tree exists) and compiles the reference's
    own programs into oracle/_ref (oracle/build_ref.sh)."""
    if not stage_ref():
        return False
    r = subprocess.run(["sh", str(HERE / "build_ref.sh")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle/build_ref.sh failed: {r.stdout[-500:]} {r.stderr[-1500:]}")
    return ref_available()


def ref_available() -> bool:
    """Whether the reference's programs are built for this machine."""
    arch = REF_DIR / "ARCH"
    if not arch.is_file() or arch.read_text().strip() != os.uname().machine:
        return False
    return all(os.access(REF_DIR / p, os.X_OK) for p in REF_PROGRAMS)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(SO))
        sig = {
            "or_bfs_serial": (_I, [_I, _P, _P, _I, _P]),
            "or_sssp_serial": (_I, [_I, _P, _P, _P, _I, _P]),
            "or_cc_serial": (_I, [_I, _P, _P, _P]),
            "or_mis_serial": (_I, [_I, _P, _P, _P]),
            "or_mis_hash": (ctypes.c_uint, [ctypes.c_uint]),
            "or_pr_f32": (_I, [_I, _P, _P, _P, _P, ctypes.c_float, _I, ctypes.c_float, _P]),
            "or_pr_f64": (_I, [_I, _P, _P, _P, _P, _I, ctypes.c_double, _I, ctypes.c_double, _P]),
            "or_pr_f64_threads": (_I, [_I, _P, _P, _P, _P, _I, ctypes.c_double, _I, ctypes.c_double, _I, _P]),
            "or_tc_serial": (ctypes.c_longlong, [_I, _P, _P]),
            "or_check_sorted": (_I, [_I, _P, _P]),
            "or_bfs_threads": (ctypes.c_double, [_I, _P, _P, _I, _P, _I]),
            "or_sssp_threads": (ctypes.c_double, [_I, _P, _P, _P, _I, _P, _I]),
            "or_cc_threads": (ctypes.c_double, [_I, _P, _P, _P, _I]),
            "or_mis_threads": (ctypes.c_double, [_I, _P, _P, _P, _I]),
            "or_pr_threads": (ctypes.c_double, [_I, _P, _P, _P, _P, ctypes.c_float, _I, ctypes.c_float, _I, _P]),
            "or_tc_threads": (ctypes.c_double, [_I, _P, _P, _P, _I]),
            "or_gen_rmat": (ctypes.c_longlong, [_I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                ctypes.c_ulonglong, _I, _I, _I, _P, _P, _P]),
            "or_degree_order": (_I, [_I, _P, _P, _P, _I, _P, _P, _P]),
            "or_pick_sources": (_I, [_I, _P, _I, ctypes.c_ulonglong, _P]),
            "or_free": (None, [_P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _arrays(g):
    nindex = np.ascontiguousarray(g.nindex, dtype=np.int32)
    nlist = np.ascontiguousarray(g.nlist, dtype=np.int32)
    return nindex, nlist


# ---------------------------------------------------------------- serial oracle
def bfs(g, src: int) -> np.ndarray:
    ni, nl = _arrays(g)
    out = np.empty(g.nodes, dtype=np.int32)
    assert lib().or_bfs_serial(g.nodes, _p(ni), _p(nl), src, _p(out)) == 0
    return out


def sssp(g, src: int) -> np.ndarray:
    ni, nl = _arrays(g)
    w = np.ascontiguousarray(g.eweight, dtype=np.int32)
    out = np.empty(g.nodes, dtype=np.int32)
    assert lib().or_sssp_serial(g.nodes, _p(ni), _p(nl), _p(w), src, _p(out)) == 0
    return out


def cc(g) -> np.ndarray:
    ni, nl = _arrays(g)
    out = np.empty(g.nodes, dtype=np.int32)
    lib().or_cc_serial(g.nodes, _p(ni), _p(nl), _p(out))
    return out


def mis(g) -> np.ndarray:
    """Status per vertex: 1 in the set, 2 excluded (reference CopyDeterm set)."""
    ni, nl = _arrays(g)
    out = np.empty(g.nodes, dtype=np.uint8)
    assert lib().or_mis_serial(g.nodes, _p(ni), _p(nl), _p(out)) > 0
    return out


def mis_hash(v: int) -> int:
    return lib().or_mis_hash(v & 0xFFFFFFFF)


def degree(g) -> np.ndarray:
    return np.diff(np.asarray(g.nindex, dtype=np.int64)).astype(np.int32)


def pr_f32(g, epsilon: float = 1e-4, max_iter: int = 100, damp: float = 0.85, scores=None):
    ni, nl = _arrays(g)
    deg = degree(g)
    s = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), dtype=np.float32) if scores is None else \
        np.array(scores, dtype=np.float32)
    res = ctypes.c_double()
    it = lib().or_pr_f32(g.nodes, _p(ni), _p(nl), _p(deg), _p(s), epsilon, max_iter, damp, ctypes.byref(res))
    return s, it, res.value


def pr_f64(g, iters: int = 0, epsilon: float = 1e-12, max_iter: int = 1000, damp: float = float(np.float32(0.85)),
           scores=None):
    ni, nl = _arrays(g)
    deg = degree(g)
    s = np.full(g.nodes, 1.0 / g.nodes, dtype=np.float64) if scores is None else np.array(scores, dtype=np.float64)
    res = ctypes.c_double()
    it = lib().or_pr_f64(g.nodes, _p(ni), _p(nl), _p(deg), _p(s), iters, epsilon, max_iter, damp, ctypes.byref(res))
    return s, it, res.value


def pr_f64_threads(g, iters: int = 0, epsilon: float = 1e-12, max_iter: int = 1000,
                   damp: float = float(np.float32(0.85)), threads: int | None = None):
    """pr_f64 with the per-vertex sums spread over host threads (same scores
    for a fixed iteration count)."""
    ni, nl = _arrays(g)
    deg = degree(g)
    s = np.full(g.nodes, 1.0 / g.nodes, dtype=np.float64)
    res = ctypes.c_double()
    it = lib().or_pr_f64_threads(g.nodes, _p(ni), _p(nl), _p(deg), _p(s), iters, epsilon, max_iter, damp,
                                 threads or os.cpu_count() or 1, ctypes.byref(res))
    return s, it, res.value


def tc(g) -> int:
    ni, nl = _arrays(g)
    return int(lib().or_tc_serial(g.nodes, _p(ni), _p(nl)))


def check_sorted(g) -> bool:
    ni, nl = _arrays(g)
    return bool(lib().or_check_sorted(g.nodes, _p(ni), _p(nl)))


# ------------------------------------------------------- threaded CPU baseline
def bfs_threads(g, src, threads):
    ni, nl = _arrays(g)
    out = np.empty(g.nodes, dtype=np.int32)
    t = lib().or_bfs_threads(g.nodes, _p(ni), _p(nl), src, _p(out), threads)
    return out, t


def sssp_threads(g, src, threads):
    ni, nl = _arrays(g)
    w = np.ascontiguousarray(g.eweight, dtype=np.int32)
    out = np.empty(g.nodes, dtype=np.int32)
    t = lib().or_sssp_threads(g.nodes, _p(ni), _p(nl), _p(w), src, _p(out), threads)
    return out, t


def cc_threads(g, threads):
    ni, nl = _arrays(g)
    out = np.empty(g.nodes, dtype=np.int32)
    t = lib().or_cc_threads(g.nodes, _p(ni), _p(nl), _p(out), threads)
    return out, t


def mis_threads(g, threads):
    ni, nl = _arrays(g)
    out = np.empty(g.nodes, dtype=np.uint8)
    t = lib().or_mis_threads(g.nodes, _p(ni), _p(nl), _p(out), threads)
    return out, t


def pr_threads(g, threads, epsilon=1e-4, max_iter=100, damp=0.85):
    ni, nl = _arrays(g)
    deg = degree(g)
    s = np.full(g.nodes, np.float32(1.0) / np.float32(g.nodes), dtype=np.float32)
    it = ctypes.c_int()
    t = lib().or_pr_threads(g.nodes, _p(ni), _p(nl), _p(deg), _p(s), epsilon, max_iter, damp, threads,
                            ctypes.byref(it))
    return s, it.value, t


def tc_threads(g, threads):
    ni, nl = _arrays(g)
    c = ctypes.c_longlong()
    t = lib().or_tc_threads(g.nodes, _p(ni), _p(nl), ctypes.byref(c), threads)
    return int(c.value), t


# ------------------------------------------------- reference programs (_ref)
def run_ref(algo: str, egr_path: str, out_path: str, threads: int = 1, src: int | None = None):
    """Runs oracle/_ref/ref_<algo>; returns the runtime the program reports."""
    exe = str(REF_DIR / f"ref_{algo}")
    args = [exe, egr_path] + ([str(src)] if src is not None else []) + [out_path, str(threads)]
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(args)} failed ({r.returncode}): {r.stderr[-500:]}")
    for line in r.stdout.splitlines():
        if line.startswith("runtime:"):
            return float(line.split()[1])
    return float("nan")


# ------------------------------------------------ workload for the CPU arms
class HostGraph:
    """ECLgraph-shaped host CSR (include/ECLgraph.h:44-50) as numpy arrays,
    for the CPU arms of the benchmark, which load no GPU library."""

    def __init__(self, nindex, nlist, eweight=None):
        self.nindex = np.ascontiguousarray(nindex, dtype=np.int32)
        self.nlist = np.ascontiguousarray(nlist, dtype=np.int32)
        self.eweight = None if eweight is None else np.ascontiguousarray(eweight, dtype=np.int32)

    @property
    def nodes(self) -> int:
        return int(self.nindex.shape[0] - 1)

    @property
    def edges(self) -> int:
        return int(self.nlist.shape[0])

    def degree(self) -> np.ndarray:
        return np.diff(self.nindex).astype(np.int32)

    def degree_ordered(self, threads: int | None = None) -> "HostGraph":
        T = threads or os.cpu_count() or 1
        ni = np.empty(self.nodes + 1, np.int32)
        nl = np.empty(max(1, self.edges), np.int32)
        ew = None if self.eweight is None else np.empty(max(1, self.edges), np.int32)
        rc = lib().or_degree_order(self.nodes, _p(self.nindex), _p(self.nlist),
                                   None if self.eweight is None else _p(self.eweight), T, _p(ni), _p(nl),
                                   None if ew is None else _p(ew))
        if rc != 0:
            raise MemoryError("or_degree_order failed")
        return HostGraph(ni, nl[:self.edges], None if ew is None else ew[:self.edges])

    def pick_sources(self, k: int, seed: int) -> np.ndarray:
        out = np.empty(k, np.int32)
        if lib().or_pick_sources(self.nodes, _p(self.nindex), k, seed, _p(out)) != 0:
            raise ValueError(f"fewer than {k} vertices with degree > 0")
        return out

    def write_egr(self, path: str) -> None:
        """The .egr byte layout of include/ECLgraph.h:82-96 (written anew)."""
        with open(path, "wb") as f:
            np.array([self.nodes, self.edges], np.int32).tofile(f)
            self.nindex.tofile(f)
            self.nlist.tofile(f)
            if self.eweight is not None:
                self.eweight.tofile(f)


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 7,
             maxw: int = 1000, permute: bool = True, threads: int | None = None) -> HostGraph:
    """The benchmark's RMAT graph, generated on the host cores by the
    oracle's copy of the generator (oracle/workload.c)."""
    T = threads or os.cpu_count() or 1
    pi, pl, pw = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    E = lib().or_gen_rmat(scale, edge_factor, a, b, c, seed, maxw, 1 if permute else 0, T, ctypes.byref(pi),
                          ctypes.byref(pl), ctypes.byref(pw))
    if E < 0:
        raise MemoryError("or_gen_rmat failed")
    n = 1 << scale
    try:
        ni = np.ctypeslib.as_array(ctypes.cast(pi, ctypes.POINTER(ctypes.c_int)), shape=(n + 1,)).copy()
        nl = np.ctypeslib.as_array(ctypes.cast(pl, ctypes.POINTER(ctypes.c_int)), shape=(max(E, 1),))[:E].copy()
        ew = None
        if maxw > 0:
            ew = np.ctypeslib.as_array(ctypes.cast(pw, ctypes.POINTER(ctypes.c_int)), shape=(max(E, 1),))[:E].copy()
    finally:
        for p in (pi, pl, pw):
            if p.value:
                lib().or_free(p)
    return HostGraph(ni, nl, ew)


class RefTimer:
    """Drives one of the reference's best-published C++ variants built as
    oracle/_ref/time_<algo> (oracle/ref/time_<algo>.cpp): the program loads
    the graph once; each run() is one call of the variant's entry function
    and returns (seconds from the variant's own timer, result summary)."""

    def __init__(self, algo: str, egr_path: str, threads: int):
        self.algo = algo
        self.p = subprocess.Popen([str(REF_DIR / f"time_{algo}"), str(egr_path), str(threads)],
                                  stdin=subprocess.PIPE, stdout=subprocess.PIPE, text=True, bufsize=1)
        for line in self.p.stdout:
            if line.startswith("ready"):
                return
        raise RuntimeError(f"time_{algo} exited before it was ready (status {self.p.wait()})")

    def run(self, src: int = 0) -> tuple:
        self.p.stdin.write(f"{int(src)}\n")
        self.p.stdin.flush()
        for line in self.p.stdout:
            if line.startswith("runtime:"):
                f = line.split()
                return float(f[1]), int(f[3])
        raise RuntimeError(f"time_{self.algo} ended during a run (status {self.p.wait()})")

    def close(self):
        if self.p.poll() is None:
            try:
                self.p.stdin.write("q\n")
                self.p.stdin.flush()
                self.p.wait(timeout=30)
            except (OSError, subprocess.TimeoutExpired):
                self.p.kill()
                self.p.wait()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
