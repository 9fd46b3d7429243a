"""CPU-only checks of the edge-list readers (prx_edge_reader_*, prx_read_mtx)
against the reference's own readers run on the same files (golden fixtures in
tests/golden/readers/, made by tests/golden/make_readers_golden.py), plus
larger seeded files checked against a numpy parse."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

READERS = os.path.join(GOLDEN, "readers")


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    pagerank_gb300.load()
    return pagerank_gb300


@pytest.fixture(scope="module")
def fx():
    z = np.load(os.path.join(READERS, "readers.npz"))
    return {k: z[k] for k in z.files}


@pytest.mark.parametrize("stem", ["temporal_small", "temporal_edge"])
def test_temporal_pieces_match_reference(pg, fx, stem):
    rows = int(fx[f"pieces_{stem}_rows"])
    with pg.graphs.EdgeReader(os.path.join(READERS, stem + ".txt")) as r:
        for i, size in enumerate(fx[f"pieces_{stem}_sizes"].tolist()):
            u, v, lines = r.next(rows, size)
            want_u, want_v = fx[f"pieces_{stem}_u{i}"], fx[f"pieces_{stem}_v{i}"]
            assert np.array_equal(u, want_u - 1), (stem, i)
            assert np.array_equal(v, want_v - 1), (stem, i)
            assert lines <= size


def test_temporal_symmetric_piece(pg, fx):
    with pg.graphs.EdgeReader(os.path.join(READERS, "temporal_small.txt")) as r:
        u, v, _ = r.next(500, 1000, symmetric=True)
    want_u, want_v = fx["pieces_temporal_small_u0"] - 1, fx["pieces_temporal_small_v0"] - 1
    assert np.array_equal(u[0::2], want_u) and np.array_equal(v[0::2], want_v)
    assert np.array_equal(u[1::2], want_v) and np.array_equal(v[1::2], want_u)


@pytest.mark.parametrize("stem", ["general", "symmetric", "skew", "rect", "array", "crlf"])
def test_mtx_matches_reference(pg, fx, stem):
    n, u, v = pg.graphs.read_mtx(os.path.join(READERS, stem + ".mtx"))
    _, rows, cols, _ = fx[f"mtx_{stem}_header"].tolist()
    assert n == max(rows, cols)
    assert np.array_equal(u, fx[f"mtx_{stem}_u"] - 1)
    assert np.array_equal(v, fx[f"mtx_{stem}_v"] - 1)


def test_pipeline_batches_are_the_lines_after_the_base_graph(pg, fx):
    """main.cu:167 then :83 -- the base graph takes the first 90% of the
    lines, each batch the next batch_fraction * size."""
    rows, size, frac = int(fx["pipe_rows"]), int(fx["pipe_size"]), float(fx["pipe_frac"])
    with pg.graphs.EdgeReader(os.path.join(READERS, "temporal_small.txt")) as r:
        u, v, lines = r.next(rows, int(0.90 * size))
        assert lines == int(0.90 * size)
        for b in range(int(fx["pipe_batches"])):
            bu, bv, _ = r.next(rows, int(frac * size))
            assert np.array_equal(bu, fx[f"pipe_raw_u{b}"] - 1)
            assert np.array_equal(bv, fx[f"pipe_raw_v{b}"] - 1)


def test_reader_errors(pg, tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("1 2\n3 9\n")
    with pg.graphs.EdgeReader(str(p)) as r:
        with pytest.raises(pg.PrxError):
            r.next(8, 10)       # id 9 > rows
    with pytest.raises(pg.PrxError):
        pg.graphs.EdgeReader(str(tmp_path / "missing.txt"))
    z = tmp_path / "zero.txt"
    z.write_text("0 1\n")
    with pg.graphs.EdgeReader(str(z)) as r:
        with pytest.raises(pg.PrxError):
            r.next(4, 1)        # ids are 1-based
    with pg.graphs.EdgeReader(str(z)) as r:   # rows == 0 or size == 0: nothing read
        assert r.next(0, 5)[2] == 0 and r.next(4, 0)[2] == 0
    e = tmp_path / "empty.mtx"
    e.write_text("")
    assert pg.graphs.read_mtx(str(e))[0] == 0


def _write_lines(path, u, v, rng):
    """u, v 1-based; random separators and a random third column."""
    sep = np.array([" ", "\t", "  "])[rng.integers(0, 3, len(u))]
    tail = np.array(["", " 7", " 123456", "\r"])[rng.integers(0, 4, len(u))]
    with open(path, "w", newline="") as f:
        f.write("".join(f"{a}{s}{b}{t}\n" for a, s, b, t in zip(u.tolist(), sep.tolist(), v.tolist(),
                                                                   tail.tolist())))


def test_large_file_in_irregular_pieces(pg, tmp_path):
    """About 6M lines (~80 MB): pieces end inside the 64 MB read buffer and
    cross its refills and the 2^20-line parse blocks."""
    rng = np.random.default_rng(5)
    rows, m = 3_000_000, 6_000_000
    u = rng.integers(1, rows + 1, m)
    v = rng.integers(1, rows + 1, m)
    path = str(tmp_path / "big.txt")
    _write_lines(path, u, v, rng)
    sizes = [1, 1_048_575, 2, 1_048_577, 2_500_000, 1_402_845, 10]
    at = 0
    with pg.graphs.EdgeReader(path) as r:
        for s in sizes:
            a, b, lines = r.next(rows, s)
            k = min(s, m - at)
            assert lines == k
            assert np.array_equal(a, u[at:at + k] - 1) and np.array_equal(b, v[at:at + k] - 1)
            at += k
    assert at == m
