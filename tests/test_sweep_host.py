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
    """The first word of every axis sets nothing, so the first variant is the
    library default; variants are the full product of the axes; every option
    a style word sets exists and accepts its value."""
    for algo, axes in sweep.STYLES.items():
        words, opts = sweep.variants(algo)[0]
        assert opts == {} and words == [next(iter(ax)) for ax in axes.values()]
        n = 1
        for vals in axes.values():
            n *= len(vals)
        assert len(sweep.variants(algo)) == n
        for words, opts in sweep.variants(algo):
            for name, value in opts.items():
                old = ig.get_option(name)
                ig.set_option(name, value)
                ig.set_option(name, old)


def test_every_other_word_leaves_the_default(ig):
    """Each word after an axis's first sets at least one option to a value
    other than the library default, so no variant repeats the default under
    another name (it would when a default moves and the axis does not)."""
    for algo, axes in sweep.STYLES.items():
        for axis, words in axes.items():
            for word, opts in list(words.items())[1:]:
                assert any(ig.get_option(k) != v for k, v in opts.items()), (algo, axis, word)


def test_style_words_name_the_axes():
    names = [sweep.variant_name("rmat20", a, w) for a in sweep.STYLES for w, _ in sweep.variants(a)]
    assert len(names) == len(set(names))
    assert "rmat20_gb300_BFS_GB300_Pull_WarpGrid_Bitmap.cu" in names
    assert "rmat20_gb300_SSSP_GB300_E_Window_Sync2_Plain_Staged_Static75.cu" in names
    assert "rmat20_gb300_TC_GB300_Item4096_Runs2_Owner.cu" in names


def test_csv_round_trip(tmp_path):
    rows = {"bfs": [(sweep.variant_name("rmat20", "bfs", ["PushPull", "WarpGrid", "Bitmap"]), 12.5),
                    (sweep.variant_name("rmat20", "bfs", ["Push", "Warp", "Dist"]), 3.25)]}
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
