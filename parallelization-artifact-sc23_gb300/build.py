"""Build recipe for the GB300 library: every translation unit under csrc/ is
compiled in parallel (nvcc for .cu with -gencode arch=compute_103a,code=sm_103a,
g++ for .cpp) and linked into indigo_gb300/libindigo_gb300.so in-tree.

Usage:  python parallelization-artifact-sc23_gb300/build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "indigo_gb300" / "libindigo_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-Wall", "-I", str(INCLUDE)] + ARCH
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off", "-I", str(INCLUDE)]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _compile(src: Path) -> Path:
    obj = OBJ / (src.name + ".o")
    newest_hdr = max((h.stat().st_mtime for h in _headers()), default=0)
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, newest_hdr):
        return obj
    if src.suffix == ".cu":
        cmd = [_nvcc(), *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    if force:
        for o in OBJ.glob("*.o"):
            o.unlink()
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [_nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


SHIM = PKG / "shim"
SHIMS = ["bfs_vertex", "sssp_vertex", "cc_vertex", "mis_vertex", "pr", "tc_vertex",
         "bfs_edge", "sssp_edge", "cc_edge", "mis_edge", "tc_edge"]


def build_shims(reference_include: str, verbose: bool = False) -> list:
    """Compiles the drop-in translation units of shim/ with the reference's
    own driver headers (include/*_cuda.h, unmodified) into _build/shim/, each
    linked against the library.  The result is the reference's driver program
    (its main, timer and verifier) running the GB300 kernels."""
    inc = Path(reference_include)
    if not (inc / "ECLgraph.h").exists():
        return []
    lib = build()
    out = OBJ / "shim"
    out.mkdir(parents=True, exist_ok=True)

    def one(name):
        exe = out / name
        src = SHIM / f"{name}_gb300.cu"
        if exe.exists() and exe.stat().st_mtime >= max(src.stat().st_mtime, lib.stat().st_mtime):
            return exe
        cmd = [_nvcc(), "-O3", "-std=c++17", *ARCH, "-w", "-include", str(SHIM / "compat_cuda13.h"),
               "-I", str(inc), "-I", str(INCLUDE), "-I", str(SHIM), str(src), "-o", str(exe),
               "-L", str(lib.parent), "-lindigo_gb300", "-Xlinker", "-rpath", "-Xlinker", str(lib.parent)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"shim build failed: {' '.join(cmd)}\n{r.stderr}")
        return exe

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        exes = list(ex.map(one, SHIMS))
    if verbose:
        print(f"built {len(exes)} drop-in driver programs in {out}")
    return exes


if __name__ == "__main__":
    # usage: build.py [--force] [reference_include_dir]
    build(force="--force" in sys.argv, verbose=True)
    inc = [a for a in sys.argv[1:] if not a.startswith("--")]
    if inc:
        build_shims(inc[0], verbose=True)
