"""Device-side graph ingest (prx_graph_create_from_edges) against the CSRs the
reference's own graph builder made: the golden graphs (tests/golden/*.npz)
from shuffled, duplicated edge lists, and main.cu's whole flow on a SNAP
temporal file (reader -> base graph with self-loops -> per batch: tidy,
apply, transpose; tests/golden/readers/readers.npz)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, load_golden
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

READERS = os.path.join(GOLDEN, "readers")


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    pagerank_gb300.load()
    return pagerank_gb300


def edges_of(off, edg):
    off = np.asarray(off, np.int64)
    u = np.repeat(np.arange(len(off) - 1, dtype=np.uint32), np.diff(off))
    return u, np.asarray(edg, np.uint32)


def assert_graph(g, off, edg, toff, tedg, tdat):
    xoff, xedg, xtoff, xtedg, xtdat = g.download()
    assert np.array_equal(xoff, off) and np.array_equal(xedg, edg)
    assert np.array_equal(xtoff, toff) and np.array_equal(xtedg, tedg)
    assert np.array_equal(xtdat, tdat)


@pytest.mark.parametrize("case", golden_cases())
def test_ingest_golden_graphs(pg, ctx, case):
    z = load_golden(case)
    n = int(z["n"])
    u, v = edges_of(z["x_off"], z["x_edg"])
    rng = np.random.default_rng(3)
    # shuffled, with a third of the edges repeated
    rep = rng.random(len(u)) < 0.33
    uu, vv = np.concatenate([u, u[rep]]), np.concatenate([v, v[rep]])
    p = rng.permutation(len(uu))
    want = (z["x_off"], z["x_edg"], z["xt_off"], z["xt_edg"], z["xt_dat"])
    g = pg.Graph.from_edges(ctx, n, uu[p], vv[p], self_loops=False)
    assert_graph(g, *want)
    g.close()
    # the golden graphs hold a self-loop on every vertex: drop them and let
    # the ingest add them back
    keep = uu[p] != vv[p]
    g = pg.Graph.from_edges(ctx, n, uu[p][keep], vv[p][keep], self_loops=True)
    assert_graph(g, *want)
    g.close()


def test_ingest_reference_pipeline(pg, ctx):
    z = np.load(os.path.join(READERS, "readers.npz"))
    z = {k: z[k] for k in z.files}
    rows, size, frac = int(z["pipe_rows"]), int(z["pipe_size"]), float(z["pipe_frac"])
    with pg.graphs.EdgeReader(os.path.join(READERS, "temporal_small.txt")) as r:
        u, v, _ = r.next(rows, int(0.90 * size))
        x = pg.Graph.from_edges(ctx, rows, u, v, self_loops=True)
        assert_graph(x, z["pipe_x_off"], z["pipe_x_edg"], z["pipe_xt_off"], z["pipe_xt_edg"], z["pipe_xt_dat"])
        xoff, xedg = z["pipe_x_off"], z["pipe_x_edg"]
        for b in range(int(z["pipe_batches"])):   # each batch applies to the graph the last one made
            bu, bv, _ = r.next(rows, int(frac * size))
            du, dv, iu, iv = x.tidy_batch([], [], bu, bv)
            assert np.array_equal(iu, z[f"pipe_ins_u{b}"] - 1) and np.array_equal(iv, z[f"pipe_ins_v{b}"] - 1)
            y = pg.Graph.from_edges(ctx, rows, *edges_of(xoff, xedg), self_loops=False)
            y.apply_batch(du, dv, iu, iv)
            assert_graph(y, z[f"pipe_y{b}_off"], z[f"pipe_y{b}_edg"], z[f"pipe_yt{b}_off"], z[f"pipe_yt{b}_edg"],
                         z[f"pipe_yt_dat{b}"])
            # the same graph straight from the edge list of x plus the batch
            xu, xv = edges_of(xoff, xedg)
            y2 = pg.Graph.from_edges(ctx, rows, np.concatenate([xu, bu]), np.concatenate([xv, bv]),
                                     self_loops=False)
            assert_graph(y2, z[f"pipe_y{b}_off"], z[f"pipe_y{b}_edg"], z[f"pipe_yt{b}_off"],
                         z[f"pipe_yt{b}_edg"], z[f"pipe_yt_dat{b}"])
            x.close()
            y2.close()
            x, (xoff, xedg) = y, (z[f"pipe_y{b}_off"], z[f"pipe_y{b}_edg"])
        x.close()


def numpy_csr(n, u, v, self_loops):
    u, v = np.asarray(u, np.uint64), np.asarray(v, np.uint64)
    if self_loops:
        s = np.arange(n, dtype=np.uint64)
        u, v = np.concatenate([u, s]), np.concatenate([v, s])
    k = np.unique(u * np.uint64(n) + v) if len(u) else np.zeros(0, np.uint64)
    su, sv = (k // np.uint64(n)).astype(np.uint32), (k % np.uint64(n)).astype(np.uint32)
    off = np.zeros(n + 1, np.uint32)
    np.cumsum(np.bincount(su, minlength=n), out=off[1:])
    toff, tedg, tdat = O.transpose(off, sv)
    return off, sv, toff, tedg, tdat


@pytest.mark.parametrize("n,m,self_loops", [(1, 0, True), (1, 5, False), (7, 0, False), (1000, 30000, True),
                                            (65537, 2_500_000, True), (300_001, 4_000_000, False)])
def test_ingest_random_vs_numpy(pg, ctx, n, m, self_loops):
    rng = np.random.default_rng(n + m)
    # skewed sources (a few long rows) and a band of isolated high ids
    hi = max(1, int(n * 0.9))
    u = np.minimum(rng.zipf(1.6, m) - 1, hi - 1).astype(np.uint32)
    v = rng.integers(0, hi, m).astype(np.uint32)
    g = pg.Graph.from_edges(ctx, n, u, v, self_loops=self_loops)
    assert_graph(g, *numpy_csr(n, u, v, self_loops))
    assert g.size() == (n, int(numpy_csr(n, u, v, self_loops)[0][-1]))
    g.close()


def test_ingest_from_device_edges(pg, ctx):
    import torch
    rng = np.random.default_rng(11)
    n, m = 50_000, 800_000
    u = rng.integers(0, n, m).astype(np.uint32)
    v = rng.integers(0, n, m).astype(np.uint32)
    du = torch.from_numpy(u.view(np.int32)).cuda()
    dv = torch.from_numpy(v.view(np.int32)).cuda()
    g = pg.Graph.from_device_edges(ctx, n, du, dv, self_loops=True)
    assert_graph(g, *numpy_csr(n, u, v, True))
    g.close()
    assert torch.equal(du.cpu(), torch.from_numpy(u.view(np.int32)))   # inputs left unchanged


def test_ingest_solves_like_host_built_graph(pg, ctx):
    off, edg = pg.graphs.rmat(12, 16, seed=9)
    u, v = edges_of(off, edg)
    p = np.random.default_rng(1).permutation(len(u))
    g = pg.Graph.from_edges(ctx, len(off) - 1, u[p], v[p], self_loops=False)
    r, res = pg.pagerank_static(ctx, g)
    want, it = O.solve("static", None, None, *O.transpose(off, edg))
    assert res["iterations"] == it and np.array_equal(r, want)
    g.close()


def test_ingest_errors(pg, ctx):
    with pytest.raises(pg.PrxError):
        pg.Graph.from_edges(ctx, 10, [1, 2, 10], [3, 4, 5])     # id 10 >= n
    with pytest.raises(pg.PrxError):
        pg.Graph.from_edges(ctx, 0, [0], [0])
    g = pg.Graph.from_edges(ctx, 0, [], [], self_loops=True)   # empty graph
    assert g.size() == (0, 0)
    g.close()
    g = pg.Graph.from_edges(ctx, 4, [1], [2])                 # context still usable after the errors
    assert g.size() == (4, 5)
    g.close()


def test_experiment_driver_runs_main_cu_flow(pg):
    """python -m pagerank_gb300.experiment on the temporal fixture: graph
    sizes as the reference's builder gives them, one result line per technique
    and batch in main.cu's format, every error small."""
    from pagerank_gb300 import experiment, report
    z = np.load(os.path.join(READERS, "readers.npz"))
    lines = experiment.run(os.path.join(READERS, "temporal_small.txt"), int(z["pipe_rows"]), int(z["pipe_size"]),
                           float(z["pipe_frac"]), batches=int(z["pipe_batches"]), partition=True, out=lambda s: None)
    text = "\n".join(lines)
    assert f"size: {len(z['pipe_x_edg'])} [directed] {{}} (selfLoopAllVertices)" in text
    for b in range(int(z["pipe_batches"])):
        assert f"size: {len(z[f'pipe_y{b}_edg'])} [directed] {{}} (insertions={len(z[f'pipe_ins_u{b}'])})" in text
    rows = report.parse_log(text)
    assert len(rows) == 10 * int(z["pipe_batches"])
    assert {r["technique"] for r in rows} == {t + p for t, _ in experiment.TECHNIQUES for p in ("", "Partition")}
    for r in rows:   # L1 over 500 vertices; tolerance 1e-10 (L-inf), frontier / prune tolerances 1e-6
        assert r["error"] < (1e-6 if "Frontier" not in r["technique"] else 1e-5) and r["iterations"] >= 1, r


# ---- edge-list text parsed on the device --------------------------------------

def graph_of(pg, ctx, n, u, v, self_loops):
    g = pg.Graph.from_edges(ctx, n, u, v, self_loops=self_loops)
    d = g.download()
    g.close()
    return d


def same_graph(g, want):
    got = g.download()
    g.close()
    assert all(np.array_equal(a, b) for a, b in zip(got, want))


@pytest.mark.parametrize("stem", ["temporal_small", "temporal_edge"])
def test_device_parse_pieces_match_host_reader(pg, ctx, stem):
    """prx_edge_reader_next_graph reads the same lines as prx_edge_reader_next,
    piece by piece, bad lines included (the fixtures are pinned to the
    reference's readTemporalDo)."""
    z = np.load(os.path.join(READERS, "readers.npz"))
    rows = int(z[f"pieces_{stem}_rows"])
    path = os.path.join(READERS, stem + ".txt")
    with pg.graphs.EdgeReader(path) as rh, pg.graphs.EdgeReader(path) as rd:
        for i, size in enumerate(z[f"pieces_{stem}_sizes"].tolist()):
            u, v, lines = rh.next(rows, size)
            assert np.array_equal(u, z[f"pieces_{stem}_u{i}"] - 1)
            g, dlines = pg.Graph.from_reader(ctx, rd, rows, size, self_loops=False)
            assert dlines == lines, (i, dlines, lines)
            same_graph(g, graph_of(pg, ctx, rows, u, v, False))


def test_device_parse_reference_pipeline(pg, ctx):
    z = np.load(os.path.join(READERS, "readers.npz"))
    rows, size = int(z["pipe_rows"]), int(z["pipe_size"])
    with pg.graphs.EdgeReader(os.path.join(READERS, "temporal_small.txt")) as r:
        g, lines = pg.Graph.from_reader(ctx, r, rows, int(0.90 * size), self_loops=True)
    assert lines == int(0.90 * size)
    same_graph(g, (z["pipe_x_off"], z["pipe_x_edg"], z["pipe_xt_off"], z["pipe_xt_edg"], z["pipe_xt_dat"]))
    text = open(os.path.join(READERS, "temporal_small.txt"), "rb").read()
    g, lines, used = pg.Graph.from_text(ctx, text, rows, int(0.90 * size), self_loops=True)
    assert lines == int(0.90 * size) and text[:used].count(b"\n") == lines
    same_graph(g, (z["pipe_x_off"], z["pipe_x_edg"], z["pipe_xt_off"], z["pipe_xt_edg"], z["pipe_xt_dat"]))


@pytest.mark.parametrize("stem", ["general", "symmetric", "skew", "rect", "array", "crlf"])
def test_device_parse_mtx(pg, ctx, stem):
    path = os.path.join(READERS, stem + ".mtx")
    n, u, v = pg.graphs.read_mtx(path)
    g, gn = pg.Graph.from_mtx(ctx, path, self_loops=True)
    assert gn == n
    same_graph(g, graph_of(pg, ctx, n, u, v, True))


def test_device_parse_large_text(pg, ctx):
    """~6M lines (~75 MB: more than the reader's 64 MB buffer), read whole and
    in irregular pieces, against the edges themselves."""
    rng = np.random.default_rng(8)
    rows, m = 2_000_000, 6_000_000
    u = rng.integers(0, rows, m).astype(np.uint32)
    v = rng.integers(0, rows, m).astype(np.uint32)
    text = pg.graphs.format_edges(u, v)
    g, lines, used = pg.Graph.from_text(ctx, text, rows, None, self_loops=True)
    assert lines == m and used == len(text)
    same_graph(g, numpy_csr(rows, u, v, True))
    p = os.path.join(os.environ.get("TMPDIR", "/tmp"), f"prx_big_{os.getpid()}.txt")
    with open(p, "wb") as f:
        f.write(text)
    try:
        at = 0
        with pg.graphs.EdgeReader(p) as r:
            for s in (1, 2_500_000, 3, 3_400_000, 1000):
                g, lines = pg.Graph.from_reader(ctx, r, rows, s, self_loops=False)
                k = min(s, m - at)
                assert lines == k
                same_graph(g, numpy_csr(rows, u[at:at + k], v[at:at + k], False))
                at += k
    finally:
        os.unlink(p)


def test_device_parse_edge_cases(pg, ctx):
    g, lines, used = pg.Graph.from_text(ctx, b"", 5, None)
    assert lines == 0 and used == 0 and g.size() == (5, 5)
    g.close()
    g, lines, used = pg.Graph.from_text(ctx, b"1 2\n3 4", 4, None, self_loops=False)   # no final newline
    assert lines == 2 and used == 7
    same_graph(g, graph_of(pg, ctx, 4, [0, 2], [1, 3], False))
    g, lines, used = pg.Graph.from_text(ctx, b"1 2\nx\n3 4\n", 4, None, self_loops=False)
    assert lines == 2 and used == 6                                                    # stops after "x"
    same_graph(g, graph_of(pg, ctx, 4, [0], [1], False))
    g, lines, used = pg.Graph.from_text(ctx, b"1 2\n3 4\n", 4, 1, self_loops=False)
    assert lines == 1 and used == 4
    g.close()
    g, lines, used = pg.Graph.from_text(ctx, b"1 2\n", 0, None)                        # rows == 0: nothing read
    assert lines == 0 and g.size() == (0, 0)
    g.close()
    with pytest.raises(pg.PrxError):
        pg.Graph.from_text(ctx, b"1 2\n3 9\n", 8, None)                                # id 9 > rows
    g, lines, _ = pg.Graph.from_text(ctx, b"1 2\n3 x\n3 9\n", 8, None, self_loops=False)   # id 9 after the stop
    assert lines == 2
    g.close()
