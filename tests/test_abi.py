"""C-ABI checks that need no GPU: the library loads, exports every function
include/indigo_gb300.h declares, and rejects bad arguments before touching
the device."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "indigo_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(ig_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_parses():
    names = declared_functions()
    assert "ig_bfs_vertex" in names and "ig_pr" in names and "ig_tc_vertex" in names
    assert len(names) > 50


def test_every_declared_symbol_is_exported(ig):
    L = ctypes.CDLL(str(ig.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert missing == []


def test_python_binding_covers_header(ig):
    from indigo_gb300._lib import SIGNATURES
    assert sorted(set(declared_functions()) - set(SIGNATURES)) == []


def test_version_and_status_strings(ig):
    L = ig.load()
    assert L.ig_version() == 1
    assert L.ig_status_string(0) == b"ok"
    assert b"sorted" in L.ig_status_string(5)
    assert L.ig_status_string(999) == b"unknown status"


def test_options_roundtrip(ig):
    old = ig.get_option("bfs_alpha")
    ig.set_option("bfs_alpha", 20)
    assert ig.get_option("bfs_alpha") == 20
    ig.set_option("bfs_alpha", old)
    with pytest.raises(ig.IndigoError):
        ig.set_option("no_such_option", 1)
    with pytest.raises(ig.IndigoError):
        ig.set_option("blocks_per_sm", 1000)


def test_kernel_option_defaults_and_ranges(ig):
    """The scheduling and work-split knobs have the measured defaults, accept
    their range and refuse values outside it (the work-item size is capped
    so a round's slice count stays small; shares are percentages)."""
    defaults = {"sssp_item_edges": 128, "sssp_warp_degree": 64, "sssp_window_scale": 8,
                "sssp_window_degree": 16, "sssp_stage_flags": 1, "sssp_static_pct": 75,
                "sssp_chunk": 32, "sssp_item_group": 8, "sssp_tail_split": 1, "sssp_claim_ahead": 0,
                "sssp_expanded_check": 0,
                "mis_static_pct": 0, "pr_blocks_per_sm": 4, "pr_static_pct": 0, "tc_block_chunk": 4096,
                "tc_grab": 2, "tc_warp_list": 64, "bfs_bu_claim": 0, "cc_bfs_seed": 1, "cc_bfs_levels": 8,
                "bfs_hub_degree": 32, "hub_degree": 256, "pr_subwarp": 1, "pr_prefetch": 0}
    for name, value in defaults.items():
        assert ig.get_option(name) == value, name
    for name, ok, bad in [("sssp_item_edges", 4096, 4097), ("sssp_item_edges", 32, 31),
                          ("sssp_window_scale", 0, -1), ("sssp_window_degree", 0, -1),
                          ("sssp_static_pct", 100, 101), ("pr_static_pct", 0, -1), ("sssp_chunk", 32, 33),
                          ("sssp_item_group", 1, 0), ("tc_warp_list", 1, 0), ("bfs_bu_claim", 64, 65)]:
        old = ig.get_option(name)
        try:
            ig.set_option(name, ok)
            assert ig.get_option(name) == ok
            with pytest.raises(ig.IndigoError):
                ig.set_option(name, bad)
            assert ig.get_option(name) == ok
        finally:
            ig.set_option(name, old)


def test_dropins_reject_bad_arguments_without_device(ig):
    L = ig.load()
    t = ctypes.c_double()
    out = np.zeros(4, np.int32)
    assert L.ig_bfs_vertex(0, None, out.ctypes.data, ctypes.byref(t)) == ig._lib.IG_ERR_INVALID_ARG
    c = ig.CSR()
    c.nodes, c.edges = 0, 0
    assert L.ig_cc_vertex(ctypes.byref(c), out.ctypes.data, ctypes.byref(t)) == ig._lib.IG_ERR_INVALID_ARG
    g = ig.grid2d(2, 2)
    hc = g.csr()
    # source out of range is refused before any device work
    assert L.ig_bfs_vertex(7, ctypes.byref(hc), out.ctypes.data, ctypes.byref(t)) == ig._lib.IG_ERR_INVALID_ARG
    assert b"source" in L.ig_last_error()
    # SSSP needs weights
    assert L.ig_sssp_vertex(0, ctypes.byref(hc), out.ctypes.data, ctypes.byref(t)) == ig._lib.IG_ERR_INVALID_ARG
    assert L.ig_pr(None, out.ctypes.data, None, 1e-4, 100, None, None) == ig._lib.IG_ERR_INVALID_ARG
    assert L.ig_tc_vertex(None, 4, None, None, None) == ig._lib.IG_ERR_INVALID_ARG


def test_every_option_is_documented_and_settable(ig):
    """Every field of the options struct (csrc/ig_options.h) is accepted by
    ig_get_option with the default the integration table states, and is
    named in the header's option list."""
    import re
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    fields = re.findall(r"^\s*(?:int|long long)\s+(\w+);", (root / "parallelization-artifact-sc23_gb300" / "csrc" /
                                                           "ig_options.h").read_text(), re.M)
    assert len(fields) > 30
    header = (root / "include" / "indigo_gb300.h").read_text()
    knobs = header[header.index("Kernel tuning knobs"):header.index("int ig_set_option")]
    table = dict(re.findall(r"^\| `(\w+)` \| (-?\d+) \|", (root / "INTEGRATION.md").read_text(), re.M))
    for name in fields:
        assert re.search(r"\b%s\b" % name, knobs), name
        assert name in table, name
        assert ig.get_option(name) == int(table[name]), name
