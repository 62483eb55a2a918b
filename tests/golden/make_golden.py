"""Generates tests/golden/golden.npz: outputs of the reference's OWN C++
programs (compiled from its sources into oracle/_ref by oracle/build_ref.sh)
on small deterministic graphs made by the library's generators.

Run in a container that has the reference tree:
    python tests/golden/make_golden.py
The fixtures pin both the oracle restatement (CPU tests) and the GPU kernels
(GPU tests) to the reference's behaviour.  Graphs are keyed by their digest so
a generator change is caught before any comparison."""
from __future__ import annotations

import hashlib
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "parallelization-artifact-sc23_gb300"))
sys.path.insert(0, str(ROOT))

import indigo_gb300 as ig  # noqa: E402
from oracle import oracle  # noqa: E402

# name -> (factory, sources); small enough to store full vectors
GRAPHS = {
    "grid64": (lambda: ig.grid2d(64, 64, maxw=255, seed=1), [0, 2080, 4095]),
    "rmat12": (lambda: ig.rmat(12, 16, seed=7, maxw=1000), None),
    "road64": (lambda: ig.road(64, 64, 0.05, 0.001, seed=11, maxw=10000), [0, 1000, 4000]),
    "er4k": (lambda: ig.erdos_renyi(4000, 8.0, seed=13, maxw=255), [0, 17, 3999]),
    "rmat12_dord": (lambda: ig.rmat(12, 16, seed=7, maxw=1000).degree_ordered(), None),
}
# the 256x256 grid of the first benchmark configuration: digests only
DIGEST_ONLY = {
    "grid256": (lambda: ig.grid2d(256, 256, maxw=255, seed=1), [0, 32896, 65535]),
}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_all(name, g, sources, tmp):
    egr = str(Path(tmp) / f"{name}.egr")
    g.write_egr(egr)
    out = {}

    def rd(path, dtype):
        return np.fromfile(path, dtype=dtype)

    if sources is None:
        sources = [int(s) for s in g.pick_sources(3, seed=7)]
    out["sources"] = np.array(sources, dtype=np.int32)
    for k, s in enumerate(sources):
        p = str(Path(tmp) / f"{name}_bfs{k}")
        oracle.run_ref("bfs", egr, p, threads=4, src=s)
        out[f"bfs{k}"] = rd(p, np.int32)
        p = str(Path(tmp) / f"{name}_sssp{k}")
        oracle.run_ref("sssp", egr, p, threads=4, src=s)
        out[f"sssp{k}"] = rd(p, np.int32)
    p = str(Path(tmp) / f"{name}_cc")
    oracle.run_ref("cc", egr, p, threads=4)
    out["cc"] = rd(p, np.int32)
    p = str(Path(tmp) / f"{name}_mis")
    oracle.run_ref("mis", egr, p, threads=4)
    out["mis"] = rd(p, np.uint8)
    p = str(Path(tmp) / f"{name}_pr")
    oracle.run_ref("pr", egr, p, threads=1)  # one thread: serial error summation order
    out["pr"] = rd(p, np.float32)
    p = str(Path(tmp) / f"{name}_tc")
    oracle.run_ref("tc", egr, p, threads=1)
    out["tc"] = rd(p, np.int64)
    return out


def main():
    if not oracle.build_ref():
        sys.exit("reference sources neither present nor staged: cannot regenerate golden fixtures")
    arrays = {}
    meta = {"graphs": {}, "digest_only": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (make, sources) in GRAPHS.items():
            g = make()
            res = run_all(name, g, sources, tmp)
            meta["graphs"][name] = {"digest": str(g.digest()), "nodes": g.nodes, "edges": g.edges}
            for k, v in res.items():
                arrays[f"{name}/{k}"] = v
            print(name, g.nodes, g.edges, "tc", int(res["tc"][0]), "mis", int((res["mis"] == 1).sum()))
        for name, (make, sources) in DIGEST_ONLY.items():
            g = make()
            res = run_all(name, g, sources, tmp)
            meta["digest_only"][name] = {
                "digest": str(g.digest()), "nodes": g.nodes, "edges": g.edges,
                "sources": [int(s) for s in res["sources"]],
                "sha256": {k: sha(v) for k, v in res.items() if k != "sources"},
                "max": {k: int(v.max()) for k, v in res.items() if k.startswith(("bfs", "sssp"))},
                "mis_size": int((res["mis"] == 1).sum()), "tc": int(res["tc"][0]),
            }
            print(name, g.nodes, g.edges, meta["digest_only"][name]["mis_size"])
    np.savez_compressed(Path(__file__).with_name("golden.npz"), **arrays)
    Path(__file__).with_name("golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
