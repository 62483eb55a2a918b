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
    src = HERE / "indigo_oracle.c"
    if force or not SO.exists() or SO.stat().st_mtime < src.stat().st_mtime:
        tmp = SO.with_suffix(".so.tmp")
        cmd = [os.environ.get("CC", "gcc"), "-O3", "-fPIC", "-shared", "-pthread", "-std=c11",
               "-ffp-contract=off", "-D_POSIX_C_SOURCE=200809L", str(src), "-o", str(tmp), "-lm"]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        os.replace(tmp, SO)
    return SO


def build_ref(reference_root: str | None = None) -> bool:
    """Builds oracle/_ref from the reference sources when they are present."""
    root = reference_root or os.environ.get("INDIGO_REFERENCE", "/root/reference")
    if not (Path(root) / "include").is_dir():
        return False
    subprocess.run(["sh", str(HERE / "build_ref.sh"), root], check=True, capture_output=True, text=True)
    return ref_available()


def reference_tree_present(reference_root: str | None = None) -> bool:
    """Whether the reference sources are on this machine (build_ref can run)."""
    root = reference_root or os.environ.get("INDIGO_REFERENCE", "/root/reference")
    return os.path.isdir(os.path.join(root, "include"))


def ref_available() -> bool:
    return all(os.access(REF_DIR / f"ref_{a}", os.X_OK) for a in ("bfs", "sssp", "cc", "mis", "pr", "tc"))


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
            "or_tc_serial": (ctypes.c_longlong, [_I, _P, _P]),
            "or_check_sorted": (_I, [_I, _P, _P]),
            "or_bfs_threads": (ctypes.c_double, [_I, _P, _P, _I, _P, _I]),
            "or_sssp_threads": (ctypes.c_double, [_I, _P, _P, _P, _I, _P, _I]),
            "or_cc_threads": (ctypes.c_double, [_I, _P, _P, _P, _I]),
            "or_mis_threads": (ctypes.c_double, [_I, _P, _P, _P, _I]),
            "or_pr_threads": (ctypes.c_double, [_I, _P, _P, _P, _P, ctypes.c_float, _I, ctypes.c_float, _I, _P]),
            "or_tc_threads": (ctypes.c_double, [_I, _P, _P, _P, _I]),
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
