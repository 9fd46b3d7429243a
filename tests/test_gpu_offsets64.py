"""64-bit offsets (prx_graph_create64): rows cut into segments whose edges are
addressed relative to the segment's start.  Small graphs with the segment
size forced down (down to 2 rows per segment) must give bit-identical ranks,
iterations and marking to the plain CSR in every mode; the bench checks a
graph of 7.6 billion edges (four copies of the 1.9B-edge graph: exactly a
quarter of one copy's ranks)."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

MODES = ["static", "naive_dynamic", "dynamic_traversal", "dynamic_frontier", "prune_dynamic_frontier"]


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    pagerank_gb300.load()
    return pagerank_gb300


def graph64(pg, ctx, yoff, yedg, yt, shift):
    return pg.Graph.from_csr64(ctx, np.asarray(yt[0], np.uint64), yt[1], yt[2], np.asarray(yoff, np.uint64), yedg,
                               seg_shift=shift)


@pytest.mark.parametrize("case", golden_cases())
@pytest.mark.parametrize("shift", [1, 3, 6])
def test_segmented_rows_bit_exact_golden(pg, ctx, case, shift):
    z = load_golden(case)
    yoff, yedg = z["y_off"], z["y_edg"]
    yt = (z["yt_off"], z["yt_edg"], z["yt_dat"])
    batch = ((z["del_u"], z["del_v"]), (z["ins_u"], z["ins_v"]))
    q = z["static_x_ranks"]
    plain = pg.Graph(ctx, *yt, yoff, yedg)
    seg = graph64(pg, ctx, yoff, yedg, yt, shift)
    for mode in MODES:
        a, ra = pg.solve(ctx, plain, pg.MODES[mode], *batch, q)
        b, rb = pg.solve(ctx, seg, pg.MODES[mode], *batch, q)
        assert ra["iterations"] == rb["iterations"] and np.array_equal(a, b), (case, shift, mode)
    for mode in ("dynamic_frontier", "dynamic_traversal"):
        fa = pg.mark_affected(ctx, plain, pg.MODES[mode], *batch)
        fb = pg.mark_affected(ctx, seg, pg.MODES[mode], *batch)
        assert np.array_equal(fa, fb)
    # the download gives the graph back, in 64-bit and 32-bit offsets
    got = seg.download64()
    assert np.array_equal(got[0], yoff) and np.array_equal(got[1], yedg)
    assert np.array_equal(got[2], yt[0]) and np.array_equal(got[3], yt[1]) and np.array_equal(got[4], yt[2])
    got32 = seg.download()
    assert np.array_equal(got32[0], yoff) and np.array_equal(got32[3], yt[1])
    plain.close()
    seg.close()


@pytest.mark.parametrize("kind", ["rmat", "web", "grid"])
@pytest.mark.parametrize("shift", [4, 10, 14])
def test_segmented_rows_synthetic(pg, ctx, kind, shift):
    """Rows of every in-degree class (thread, warp, block kernels) across
    segment boundaries; Static, DF-P and the FP32 refinement."""
    if kind == "rmat":
        xoff, xedg = pg.graphs.rmat(15, 16, seed=4)
    elif kind == "web":
        xoff, xedg = pg.graphs.weblike(200_000, seed=4)
    else:
        xoff, xedg = pg.graphs.grid(200, seed=4)
    batch = pg.graphs.random_batch(xoff, xedg, 200, 800, seed=2)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    plain = pg.Graph(ctx, *yt, yoff, yedg)
    seg = graph64(pg, ctx, yoff, yedg, yt, shift)
    q, _ = pg.pagerank_static(ctx, pg.Graph.from_out_csr(ctx, xoff, xedg))
    for mode in ("static", "prune_dynamic_frontier", "dynamic_traversal"):
        a, ra = pg.solve(ctx, plain, pg.MODES[mode], batch[:2], batch[2:], q)
        b, rb = pg.solve(ctx, seg, pg.MODES[mode], batch[:2], batch[2:], q)
        assert ra["iterations"] == rb["iterations"] and np.array_equal(a, b), (kind, shift, mode)
    o32 = pg.options(precision=pg.FP32_REFINE)
    a, ra = pg.solve(ctx, plain, pg.STATIC, opts=o32)
    b, rb = pg.solve(ctx, seg, pg.STATIC, opts=o32)
    assert ra["iterations"] == rb["iterations"] and np.array_equal(a, b)
    # source chunks: one layout per row segment (segments of 32 rows or more);
    # 7 chunks (the coalesced scatter) and 20 (the general one)
    n = len(yoff) - 1
    for width in (n // 7 + 1, n // 20 + 1):
        for mode in ("static", "prune_dynamic_frontier"):
            for prec in (pg.FP64, pg.FP32_REFINE):
                o = pg.options(chunk_vertices=width, precision=prec)
                b, rb = pg.solve(ctx, seg, pg.MODES[mode], batch[:2], batch[2:], q, o)
                a, ra = pg.solve(ctx, plain, pg.MODES[mode], batch[:2], batch[2:], q, o)
                assert ra["iterations"] == rb["iterations"] and np.array_equal(a, b), (kind, shift, width, mode)
    plain.close()
    seg.close()


def test_segmented_rows_limits(pg, ctx):
    xoff, xedg = pg.graphs.rmat(10, 8, seed=1)
    xt = O.transpose(xoff, xedg)
    auto = graph64(pg, ctx, xoff, xedg, xt, 0)          # m < 2^32: one segment, the plain CSR
    r, res = pg.pagerank_static(ctx, auto)
    want, it = O.solve("static", None, None, *xt)
    assert res["iterations"] == it and np.array_equal(r, want)
    auto.apply_batch(*pg.graphs.random_batch(xoff, xedg, 5, 5, seed=1))   # plain: batches work
    auto.close()
    seg = graph64(pg, ctx, xoff, xedg, xt, 5)
    e = np.zeros(0, np.uint32)
    for call in (lambda: seg.apply_batch(e, e, e, e), lambda: seg.tidy_batch(e, e, e, e),
                 lambda: seg.gen_batch(1, 1), lambda: pg.solve_ppr_batched(ctx, seg, [[0]])):
        with pytest.raises(pg.PrxError) as err:
            call()
        assert err.value.status == 5   # PRX_ERANGE
    seg.close()
    with pytest.raises(pg.PrxError):
        graph64(pg, ctx, xoff, xedg, xt, 33)
