"""Variant-sweep harness, host side: the first variant of every algorithm is
the library default, and its tables round-trip in the reference's layout
(a quoted "filename" column whose names end in a newline, and a throughput
column)."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "parallelization-artifact-sc23_gb300"))

import sweep  # noqa: E402


def test_first_variant_is_the_default(ig):
    for algo, axes in sweep.AXES.items():
        first = sweep.variants(algo)[0]
        for name, value in first.items():
            assert ig.get_option(name) == value, (algo, name)
        n = 1
        for vals in axes.values():
            n *= len(vals)
        assert len(sweep.variants(algo)) == n


def test_csv_round_trip(tmp_path):
    rows = {"bfs": [(sweep.variant_name("rmat20", "bfs", {"blocks_per_sm": 4, "hub_degree": 256}), 12.5),
                    (sweep.variant_name("rmat20", "bfs", {"blocks_per_sm": 2, "hub_degree": 64}), 3.25)]}
    p = tmp_path / "t.csv"
    sweep.write_csv(str(p), rows)
    text = p.read_text()
    assert text.startswith('"filename","bfs"')
    back = sweep.read_reference_csv(str(p))
    assert [(n, round(v, 6)) for n, v in back] == [(n, v) for n, v in rows["bfs"]]
    # a row in the reference's own quoting (name, newline inside the quotes)
    q = tmp_path / "ref.csv"
    q.write_text('"filename","bfs"\n"rmat_x_BFS_CUDA_V_Data_Push.cu\n","0.399387"\n')
    assert sweep.read_reference_csv(str(q)) == [("rmat_x_BFS_CUDA_V_Data_Push.cu", 0.399387)]
