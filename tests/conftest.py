"""Test configuration: puts the package and the oracle on sys.path, builds
the library / oracle when missing, registers the `gpu` marker."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "parallelization-artifact-sc23_gb300"
for p in (str(PKG), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: full-size workloads")


def _ensure_built():
    import build as pkg_build  # parallelization-artifact-sc23_gb300/build.py
    pkg_build.build()
    from oracle import oracle
    oracle.build()


_ensure_built()


@pytest.fixture(scope="session")
def ig():
    import indigo_gb300
    return indigo_gb300


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def golden():
    meta = json.loads((GOLDEN / "golden.json").read_text())
    arrays = dict(np.load(GOLDEN / "golden.npz"))
    return meta, arrays


@pytest.fixture(scope="session")
def gpu(ig):
    if ig.device_count() < 1:
        pytest.fail("no CUDA device visible to a test marked gpu")
    return True


def golden_graphs(ig):
    """The generators behind the golden fixtures (same parameters)."""
    return {
        "grid64": lambda: ig.grid2d(64, 64, maxw=255, seed=1),
        "rmat12": lambda: ig.rmat(12, 16, seed=7, maxw=1000),
        "road64": lambda: ig.road(64, 64, 0.05, 0.001, seed=11, maxw=10000),
        "er4k": lambda: ig.erdos_renyi(4000, 8.0, seed=13, maxw=255),
        "rmat12_dord": lambda: ig.rmat(12, 16, seed=7, maxw=1000).degree_ordered(),
        "grid256": lambda: ig.grid2d(256, 256, maxw=255, seed=1),
    }


def kat_graphs(ig):
    """Small graphs with known answers and edge cases (built from arrays)."""
    G = ig.Graph

    def from_edges(n, edges, w=None):
        adj = [[] for _ in range(n)]
        for (u, v) in edges:
            adj[u].append(v)
            adj[v].append(u)
        nindex = [0]
        nlist = []
        for v in range(n):
            s = sorted(set(adj[v]))
            nlist += s
            nindex.append(len(nlist))
        nl = np.array(nlist, dtype=np.int32)
        ew = None
        if w:
            ew = np.array([1 + ((min(v, u) * 7 + max(v, u) * 13) % w) for v in range(n)
                           for u in nl[nindex[v]:nindex[v + 1]]], dtype=np.int32)
        return G(np.array(nindex, dtype=np.int32), nl, ew)

    k = 12
    return {
        "single": G(np.array([0, 0], np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32)),
        "two_isolated": G(np.array([0, 0, 0], np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32)),
        "edge": from_edges(2, [(0, 1)], 9),
        "path": from_edges(50, [(i, i + 1) for i in range(49)], 9),
        "star": from_edges(40, [(0, i) for i in range(1, 40)], 9),
        "complete": from_edges(k, [(i, j) for i in range(k) for j in range(i + 1, k)], 9),
        "two_grids": _disjoint_grids(ig),
        "hubby": from_edges(3000, [(0, i) for i in range(1, 3000)] + [(1, i) for i in range(2, 2600)] +
                            [(i, i + 1) for i in range(5, 2999)], 50),
    }


def _disjoint_grids(ig):
    a = ig.grid2d(10, 10, maxw=5, seed=3)
    b = ig.grid2d(7, 9, maxw=5, seed=4)
    n = a.nodes + b.nodes
    nindex = np.concatenate([a.nindex, b.nindex[1:] + a.edges]).astype(np.int32)
    nlist = np.concatenate([a.nlist, b.nlist + a.nodes]).astype(np.int32)
    ew = np.concatenate([a.eweight, b.eweight]).astype(np.int32)
    g = ig.Graph(nindex, nlist, ew)
    assert g.nodes == n
    return g
