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
    with pytest.raises(pg.PrxError):
        graph64(pg, ctx, xoff, xedg, xt, 33)


@pytest.mark.parametrize("shift", [3, 7, 12])
def test_segmented_weights_and_adjoint_bit_exact(pg, ctx, shift):
    """Edge weights, the weighted solve and the adjoint (dL/dw in the caller's
    compact out-CSR order, dL/dt, dL/dalpha) on a graph of row segments give
    the plain CSR's bits, also after a device-applied batch."""
    import torch
    from pagerank_gb300 import autograd as A
    xoff, xedg = pg.graphs.rmat(12, 16, a=0.6, b=0.15, c=0.15, seed=8)
    xt = O.transpose(xoff, xedg)
    plain = pg.Graph(ctx, *xt, xoff, xedg)
    seg = graph64(pg, ctx, xoff, xedg, xt, shift)
    rng = np.random.default_rng(shift)
    n = len(xoff) - 1
    gl = torch.from_numpy(rng.standard_normal(n)).cuda()
    t = torch.from_numpy(rng.uniform(0.5, 1.5, n) / n).cuda()
    o = pg.options(tolerance=1e-12)
    for step in range(2):
        m = plain.size()[1]
        w = torch.from_numpy(rng.uniform(0.5, 2.0, m).astype(np.float32)).cuda()
        outs = []
        for g in (plain, seg):
            A.set_weights(ctx, g, w)
            r, rr = A.solve_weighted(ctx, g, t, opts=o)
            adj = A.adjoint(ctx, g, r, gl, t, opts=o)
            outs.append((r.cpu().numpy(), rr["iterations"], adj["grad_w"].cpu().numpy(),
                         adj["grad_t"].cpu().numpy(), adj["grad_alpha"]))
        a, b = outs
        assert a[1] == b[1]
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y)), (shift, step)
        if step == 0:
            batch = plain.gen_batch(40, 160, seed=5)
            plain.apply_batch(*batch)
            seg.apply_batch(*batch)
    plain.close()
    seg.close()


def _same_graph(plain, seg):
    a, b = plain.download(), seg.download64()
    for x, y in zip(a, b):
        assert np.array_equal(np.asarray(x, np.uint64), np.asarray(y, np.uint64))


@pytest.mark.parametrize("kind,shift", [("rmat", 3), ("rmat", 5), ("rmat", 12), ("web", 4), ("web", 11),
                                        ("grid", 7)])
def test_segmented_batches_bit_exact(pg, ctx, kind, shift):
    """Batch generation, tidying and application on the device keep a graph of
    row segments identical to the plain CSR (segments move to new bases, some
    of them not on a 32-row boundary); DF-P after the device-applied batch,
    Static and batched PPR then give the plain CSR's bits."""
    if kind == "rmat":
        xoff, xedg = pg.graphs.rmat(13, 12, seed=5)
    elif kind == "web":
        xoff, xedg = pg.graphs.weblike(60_000, seed=5)
    else:
        xoff, xedg = pg.graphs.grid(120, seed=5)
    xt = O.transpose(xoff, xedg)
    plain = pg.Graph(ctx, *xt, xoff, xedg)
    seg = graph64(pg, ctx, xoff, xedg, xt, shift)
    q, _ = pg.pagerank_static(ctx, plain)
    for step in range(2):
        # the device generator draws the same batch from both layouts
        b0 = plain.gen_batch(300, 900, seed=11 + step)
        b1 = seg.gen_batch(300, 900, seed=11 + step)
        assert all(np.array_equal(x, y) for x, y in zip(b0, b1))
        # tidying a raw batch with repeats, missing deletions and existing insertions
        rng = np.random.default_rng(step)
        n = len(xoff) - 1
        raw = (np.concatenate([b0[0], b0[0][:50], rng.integers(0, n, 40)]).astype(np.uint32),
               np.concatenate([b0[1], b0[1][:50], rng.integers(0, n, 40)]).astype(np.uint32),
               np.concatenate([b0[2], b0[2][:70], b0[0][:30]]).astype(np.uint32),
               np.concatenate([b0[3], b0[3][:70], b0[1][:30]]).astype(np.uint32))
        t0, t1 = plain.tidy_batch(*raw), seg.tidy_batch(*raw)
        assert all(np.array_equal(x, y) for x, y in zip(t0, t1))
        plain.apply_batch(*t0)
        seg.apply_batch(*t0)
        _same_graph(plain, seg)
        for mode in ("prune_dynamic_frontier", "dynamic_frontier", "dynamic_traversal"):
            a, ra = pg.solve(ctx, plain, pg.MODES[mode], t0[:2], t0[2:], q)
            b, rb = pg.solve(ctx, seg, pg.MODES[mode], t0[:2], t0[2:], q)
            assert ra["iterations"] == rb["iterations"] and np.array_equal(a, b), (kind, shift, step, mode)
        q, rs = pg.pagerank_static(ctx, plain)
        q1, rs1 = pg.pagerank_static(ctx, seg)
        assert rs["iterations"] == rs1["iterations"] and np.array_equal(q, q1)
    # batched personalized PageRank (rows above low_max in segments of seg_edges)
    seeds = [[0], [1, 2, 3], list(range(0, len(xoff) - 1, 97))]
    for o in (pg.options(tolerance=1e-10), pg.options(tolerance=1e-10, precision=pg.FP32_REFINE)):
        a, ra = pg.solve_ppr_batched(ctx, plain, seeds, o)
        b, rb = pg.solve_ppr_batched(ctx, seg, seeds, o)
        assert ra["iterations"] == rb["iterations"] and np.array_equal(a, b)
    plain.close()
    seg.close()
