"""CPU-only checks: the C-ABI library loads and exports every declared entry
point, and its host utilities agree with the oracle and the golden fixtures."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_cases, load_golden
from oracle import pyoracle as O


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    pagerank_gb300.load()
    return pagerank_gb300


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^\s*(?:[\w\*]+\s+)+\**(prx_\w+)\s*\(", text, re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol(pg):
    import ctypes
    lib = ctypes.CDLL(pg.library_path())
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    from pagerank_gb300 import _lib
    assert set(_lib.EXPORTS) <= set(names)


def test_options_default(pg):
    o = pg.options()
    assert (o.repeat, o.tolerance, o.frontier_tolerance, o.prune_tolerance, o.damping, o.max_iterations) == \
           (1, 1e-10, 1e-6, 1e-6, 0.85, 500)


def _check_csr(off, edg, n):
    assert off[0] == 0 and off[-1] == len(edg) and len(off) == n + 1
    assert np.all(np.diff(off.astype(np.int64)) >= 1)          # self-loop on every vertex
    assert edg.max() < n
    for u in range(0, n, max(1, n // 200)):
        row = edg[off[u]:off[u + 1]]
        assert np.all(np.diff(row.astype(np.int64)) > 0)      # ascending, unique
        assert u in row


def test_generators_shape_and_determinism(pg):
    off, edg = pg.graphs.rmat(12, 16, seed=5)
    _check_csr(off, edg, 4096)
    off2, edg2 = pg.graphs.rmat(12, 16, seed=5)
    np.testing.assert_array_equal(off, off2)
    np.testing.assert_array_equal(edg, edg2)
    off3, _ = pg.graphs.rmat(12, 16, seed=6)
    assert not np.array_equal(off, off3)
    off, edg = pg.graphs.weblike(20000, window=64, seed=3)
    _check_csr(off, edg, 20000)
    off, edg = pg.graphs.grid(50, diag=0.05, seed=1)
    _check_csr(off, edg, 2500)
    # 4-neighbour edges: 2 * 2 * w * (w-1); plus self-loops; plus diagonal pairs
    assert len(edg) >= 2 * 2 * 50 * 49 + 2500


def test_host_transpose_matches_oracle(pg):
    off, edg = pg.graphs.rmat(11, 8, seed=9)
    got = pg.graphs.transpose(off, edg)
    want = O.transpose(off, edg)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("case", golden_cases())
def test_host_tidy_and_apply_match_reference(pg, case):
    z = load_golden(case)
    du, dv, iu, iv = pg.graphs.tidy_batch(z["x_off"], z["x_edg"], z["raw_del_u"], z["raw_del_v"],
                                          z["raw_ins_u"], z["raw_ins_v"])
    for a, k in zip((du, dv, iu, iv), ("del_u", "del_v", "ins_u", "ins_v")):
        np.testing.assert_array_equal(a, z[k])
    yoff, yedg = pg.graphs.apply_batch(z["x_off"], z["x_edg"], du, dv, iu, iv)
    np.testing.assert_array_equal(yoff, z["y_off"])
    np.testing.assert_array_equal(yedg, z["y_edg"])


def test_random_batch_is_tidy(pg):
    off, edg = pg.graphs.rmat(10, 16, seed=2)
    du, dv, iu, iv = pg.graphs.random_batch(off, edg, 50, 200, seed=4)
    assert 0 < len(du) <= 50 and 0 < len(iu) <= 200
    for u, v in zip(du, dv):
        assert u != v and v in edg[off[u]:off[u + 1]]
    for u, v in zip(iu, iv):
        assert v not in edg[off[u]:off[u + 1]]
    k = du.astype(np.uint64) << 32 | dv
    assert np.all(np.diff(k.astype(np.float64)) > 0)
    yoff, yedg = pg.graphs.apply_batch(off, edg, du, dv, iu, iv)
    y2 = O.apply_batch(off, edg, du, dv, iu, iv)
    np.testing.assert_array_equal(yoff, y2[0])
    np.testing.assert_array_equal(yedg, y2[1])


def test_status_strings(pg):
    from pagerank_gb300 import _lib
    lib = pg.load()
    for code, text in _lib.STATUS.items():
        assert lib.prx_status_string(code).decode() == text
    assert lib.prx_status_string(99).decode() == "unknown status"
