"""bench.py's host-side helpers, without a GPU: the algorithmic bytes behind
the roofline figures, the nvidia-smi clock record it parses, the measured
peaks it divides by, the DRAM figures it reports, and the PageRank error
against the FP64 oracle."""
import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["bench_under_test"] = mod
    spec.loader.exec_module(mod)
    return mod


def test_algorithmic_bytes_formulas(bench, ig):
    g = ig.rmat(10, 16, seed=7, maxw=1000, permute=True)
    gd = g.degree_ordered()
    V, E = g.nodes, g.edges
    b = bench.algorithmic_bytes(g, gd, 15)
    assert b["bfs"] == 4 * (V + 1) + 8 * E + 4 * V
    assert b["sssp"] == 12 * E + 8 * V
    assert b["cc"] == 8 * E + 8 * V
    assert b["mis"] == 8 * E + 12 * V
    assert b["pr"] == 15 * (8 * E + 20 * V)
    # TC: sum over oriented edges u -> v (v after u in (degree, id) order) of
    # 4 (d+(u) + d+(v)), plus 4E + 4V, counted here edge by edge
    ni, nl = np.asarray(gd.nindex), np.asarray(gd.nlist)
    dplus = np.array([int((nl[ni[u]:ni[u + 1]] > u).sum()) for u in range(gd.nodes)])
    tot = 0
    for u in range(gd.nodes):
        for v in nl[ni[u]:ni[u + 1]]:
            if v > u:
                tot += 4 * (dplus[u] + dplus[v])
    assert b["tc"] == tot + 4 * E + 4 * V


class _Done:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_record_parsing(bench, tmp_path):
    """Median SM clock, highest max clock and every throttle reason seen
    active, from nvidia-smi's csv rows (malformed rows are skipped)."""
    s = bench.ClockSampler.__new__(bench.ClockSampler)
    f = open(tmp_path / "clocks.csv", "w+")
    f.write("0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n"
            "0, 1980, 2070, 1350.0, 0x4, Not Active, Not Active, Not Active, Active\n"
            "0, 2070, 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active\n"
            "garbage line\n"
            "0, [N/A], 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active\n")
    f.flush()
    s.file, s.proc = f, _Done()
    r = s.stop()
    assert r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0 and r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]
    s2 = bench.ClockSampler.__new__(bench.ClockSampler)
    s2.proc = None
    assert s2.stop()["reasons"] == ["nvidia-smi unavailable"]


def test_peaks_and_dram_figures(bench):
    p = bench.load_peaks()
    assert p["hbm_gbs"] > 1000
    assert "measured" in p["source"] or "fallback" in p["source"]
    assert set(bench.DRAM_BYTES_PER_CALL) <= set(bench.ALGOS)
    assert all(v > 0 for v in bench.DRAM_BYTES_PER_CALL.values())
    assert bench.RUNS_PER_STEP == 2 * bench.N_SOURCES + 4


def test_pagerank_error_against_fp64(bench, ig, orc):
    """Scores equal to the FP64 oracle rounded to FP32 have errors at the
    FP32 rounding level against the same-iteration and converged runs."""
    g = ig.rmat(10, 16, seed=7, maxw=1000)
    ref, it, _ = orc.pr_f64(g)
    e = bench.pagerank_error(g, ref.astype(np.float32), it)
    assert e["rel_l1_vs_fp64_converged"] < 1e-7
    assert e["rel_l1_vs_fp64_same_iterations"] < 1e-6
    assert e["fp64_converged_residual"] < 1e-12
