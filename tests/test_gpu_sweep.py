"""Variant sweep on the GPU: every kernel-option variant of every algorithm
runs on a small graph and returns the same result as the default variant
(the harness raises otherwise); every variant gets a positive throughput."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "parallelization-artifact-sc23_gb300"))

import sweep  # noqa: E402

pytestmark = pytest.mark.gpu


def test_all_variants_agree(ig, gpu, tmp_path):
    g = ig.rmat(12, 16, seed=7, maxw=1000)
    rows = sweep.sweep(g, list(sweep.AXES), 1, "rmat12", log=lambda *a: None)
    for algo in sweep.AXES:
        assert len(rows[algo]) == len(sweep.variants(algo))
        assert all(v > 0 for _, v in rows[algo])
    sweep.write_csv(str(tmp_path / "s.csv"), rows)
    assert len(sweep.read_reference_csv(str(tmp_path / "s.csv"))) > 0
