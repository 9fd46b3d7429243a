"""FP64 sweeps with part of the edge additions on the integer pipes
(prx_options.int_adds 1 .. 4): the integer adder is correctly rounded, so
every mode gives the oracle's ranks and iteration counts bit for bit, with
source chunks, hot sources, both loops and the FP32 refinement's FP64
sweeps; operands outside its range (negative or huge ranks) fall back to the
FP64 add with the same bits."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

MODES = ("static", "naive_dynamic", "dynamic_traversal", "dynamic_frontier", "prune_dynamic_frontier")


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    return pagerank_gb300


def _synthetic(pg, kind):
    if kind == "rmat16":
        return pg.graphs.rmat(16, 16, seed=42)
    if kind == "web200k":
        return pg.graphs.weblike(200000, dmax=20000, window=4096, seed=42)
    if kind == "grid256":
        return pg.graphs.grid(256, 0.05, seed=42)
    return pg.graphs.rmat(14, 48, a=0.7, b=0.1, c=0.1, seed=3)   # hubs


@pytest.mark.parametrize("int_adds", [1, 2, 3, 4])
@pytest.mark.parametrize("case", golden_cases())
def test_golden_all_modes(pg, ctx, case, int_adds):
    z = load_golden(case)
    batch = (z["del_u"], z["del_v"], z["ins_u"], z["ins_v"])
    xt = (z["yt_off"], z["yt_edg"], z["yt_dat"])
    g = pg.Graph(ctx, *xt, z["y_off"], z["y_edg"], validate=True)
    q = z["static_x_ranks"]
    for mode in MODES:
        want, it_w = O.solve(mode, z["y_off"], z["y_edg"], *xt, *batch, q=q)
        got, res = pg.solve(ctx, g, pg.MODES[mode], batch[:2], batch[2:], q, pg.options(int_adds=int_adds))
        assert res["iterations"] == it_w, mode
        np.testing.assert_array_equal(got, want, err_msg=mode)
    g.close()


@pytest.mark.parametrize("kind", ["rmat16", "web200k", "grid256", "hubs"])
def test_synthetic_all_modes(pg, ctx, kind):
    xoff, xedg = _synthetic(pg, kind)
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, max(1, int(2e-5 * m)), max(1, int(8e-5 * m)), seed=11)
    xt = O.transpose(xoff, xedg)
    q, _ = O.solve("static", None, None, *xt)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    g = pg.Graph(ctx, *xt, xoff, xedg, validate=True)
    g.apply_batch(*batch)
    for mode in MODES:
        want, it_w = O.solve(mode, yoff, yedg, *yt, *batch, q=q)
        for int_adds in (1, 2, 3, 4):
            for width, loop in ((0, pg.LOOP_AUTO), (997, pg.LOOP_HOST)):
                o = pg.options(int_adds=int_adds, chunk_vertices=width, loop=loop)
                got, res = pg.solve(ctx, g, pg.MODES[mode], batch[:2], batch[2:], q, o)
                assert res["iterations"] == it_w, (kind, mode, int_adds, width)
                np.testing.assert_array_equal(got, want, err_msg=f"{kind} {mode} int_adds={int_adds}")
    # the FP32 refinement's FP64 sweeps: the same bits as without the integer adds
    for mode in ("static", "prune_dynamic_frontier"):
        ref, r0 = pg.solve(ctx, g, pg.MODES[mode], batch[:2], batch[2:], q,
                           pg.options(int_adds=-1, precision=pg.FP32_REFINE))
        for int_adds in (1, 2, 4):
            got, r1 = pg.solve(ctx, g, pg.MODES[mode], batch[:2], batch[2:], q,
                               pg.options(int_adds=int_adds, precision=pg.FP32_REFINE))
            assert r1["iterations"] == r0["iterations"]
            np.testing.assert_array_equal(got, ref)
    g.close()


def test_out_of_range_operands_fall_back(pg, ctx):
    # ranks the integer adder does not take (negative, above 2^977) reach the
    # row sums through q; the FP64 add takes those steps, with the same bits
    xoff, xedg = _synthetic(pg, "rmat16")
    xt = O.transpose(xoff, xedg)
    g = pg.Graph(ctx, *xt, xoff, xedg, validate=True)
    q, _ = O.solve("static", None, None, *xt)
    e = np.zeros(0, np.uint32)
    seed = (np.array([0], np.uint32), np.array([1], np.uint32))   # marking seeds only
    for bad in (-1e-3, 1e300):
        qb = q.copy()
        qb[::97] = bad
        for mode, ins in ((pg.NAIVE_DYNAMIC, (e, e)), (pg.DYNAMIC_FRONTIER, seed)):
            want, w = pg.solve(ctx, g, mode, (e, e), ins, qb, pg.options(max_iterations=3, int_adds=-1))
            for int_adds in (1, 2, 4):
                got, r = pg.solve(ctx, g, mode, (e, e), ins, qb, pg.options(max_iterations=3, int_adds=int_adds))
                assert r["iterations"] == w["iterations"]
                assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (bad, mode, int_adds)
    for bad in (-2, 5):
        with pytest.raises(pg.PrxError):
            pg.solve(ctx, g, pg.STATIC, opts=pg.options(int_adds=bad))
    g.close()
