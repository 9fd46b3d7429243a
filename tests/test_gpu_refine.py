"""FP32 storage with FP64 refinement (PRX_FP32_REFINE) against the FP64 oracle.

The bar is the one the design states for this path: ranks within L-inf 1e-9 of
the FP64 result at tol 1e-10, with the FP64 residual test deciding
convergence (so at most a few sweeps more than the FP64 loop)."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
LINF = 1e-9


def bound(want):
    # 1e-9 absolute is the target on the benchmark graphs (ranks ~1e-8); on the
    # tiny fixtures ranks reach 1e-2..1e-1, where FP32 spacing alone is ~1e-9
    # and two tol-converged answers differ by that much, so scale with the
    # largest rank there.
    return max(LINF, 3e-8 * float(np.max(want)))


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    return pagerank_gb300


@pytest.mark.parametrize("case", golden_cases())
def test_refine_static_and_nd_golden(pg, ctx, case):
    z = load_golden(case)
    xt = (z["yt_off"], z["yt_edg"], z["yt_dat"])
    g = pg.Graph(ctx, *xt)
    opts = pg.options(precision=pg.FP32_REFINE)
    try:
        want, it = O.solve("static", None, None, *xt)
        got, res = pg.solve(ctx, g, pg.STATIC, opts=opts)
        assert np.abs(got - want).max() <= bound(want)
        # small graphs have ranks near 1e-2..1e-1, where FP32 resolves ~1e-9:
        # the FP64 test then needs a second round of FP32 sweeps
        assert it <= res["iterations"] <= 2 * it + 10 and res["refinements"] >= 1
        q = z["static_x_ranks"]
        want, it = O.solve("naive_dynamic", None, None, *xt, q=q)
        got, res = pg.solve(ctx, g, pg.NAIVE_DYNAMIC, q=q, opts=opts)
        assert np.abs(got - want).max() <= bound(want)
        assert it <= res["iterations"] <= 2 * it + 10
    finally:
        g.close()


@pytest.mark.parametrize("kind", ["rmat16", "web200k", "hubs"])
def test_refine_static_synthetic(pg, ctx, kind):
    from test_gpu_parity import _synthetic
    xoff, xedg = _synthetic(pg, kind)
    xt = O.transpose(xoff, xedg)
    g = pg.Graph(ctx, *xt)
    try:
        want, it = O.solve("static", None, None, *xt)
        got, res = pg.solve(ctx, g, pg.STATIC, opts=pg.options(precision=pg.FP32_REFINE))
        err = np.abs(got - want).max()
        assert err <= bound(want), err
        assert it <= res["iterations"] <= 2 * it + 10
    finally:
        g.close()


def test_refine_caps_and_tolerances(pg, ctx):
    xoff, xedg = pg.graphs.rmat(12, 16, seed=3)
    xt = O.transpose(xoff, xedg)
    g = pg.Graph(ctx, *xt)
    for L in (0, 1, 2, 5):
        want, it = O.solve("static", None, None, *xt, opts=O.options(max_iterations=L))
        got, res = pg.solve(ctx, g, pg.STATIC, opts=pg.options(precision=pg.FP32_REFINE, max_iterations=L))
        assert res["iterations"] == it
        # early iterates are far from converged; FP32 storage of the correction
        # still keeps them within a relative 1e-6 of the FP64 iterate
        assert np.abs(got - want).max() <= 1e-6 * want.max()
    want, it = O.solve("static", None, None, *xt, opts=O.options(tolerance=1e-13))
    got, res = pg.solve(ctx, g, pg.STATIC, opts=pg.options(precision=pg.FP32_REFINE, tolerance=1e-13))
    assert np.abs(got - want).max() <= 1e-12
    g.close()


@pytest.mark.parametrize("kind", ["web200k", "hubs", "rmat16"])
def test_refine_dynamic_modes(pg, ctx, kind):
    # DT / DF / DF-P with FP32 ranks, then FP64 sweeps over all vertices until
    # the L-inf test passes.  The answer is the converged (Static) ranks to the
    # refinement bound; its distance from the FP64 path's answer is at most
    # that path's own distance from them (pruned vertices keep stale ranks
    # there) plus the bound.  Same initial affected set, both loops.
    from test_gpu_parity import _synthetic
    xoff, xedg = _synthetic(pg, kind)
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, max(1, int(2e-4 * m)), max(1, int(8e-4 * m)), seed=29)
    du, dv, iu, iv = batch
    xt = O.transpose(xoff, xedg)
    q, _ = O.solve("static", None, None, *xt)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    g = pg.Graph(ctx, *yt, yoff, yedg)
    try:
        conv, _ = O.solve("static", None, None, *yt)
        for mode in ("dynamic_traversal", "dynamic_frontier", "prune_dynamic_frontier"):
            want, _ = O.solve(mode, yoff, yedg, *yt, du, dv, iu, iv, q=q)
            own = np.abs(want - conv).max()
            _, r64 = pg.solve(ctx, g, pg.MODES[mode], (du, dv), (iu, iv), q)
            # the FP32 phase as the mode's own iterations (2), as full sweeps (1),
            # and picked by the size of the initial marking (0)
            for loop, sweeps in ((pg.LOOP_GRAPH, 2), (pg.LOOP_HOST, 2), (pg.LOOP_GRAPH, 1), (pg.LOOP_GRAPH, 0)):
                o = pg.options(precision=pg.FP32_REFINE, loop=loop, refine_sweeps=sweeps)
                got, res = pg.solve(ctx, g, pg.MODES[mode], (du, dv), (iu, iv), q, o)
                assert np.abs(got - conv).max() <= bound(conv), (kind, mode, loop, sweeps)
                assert np.abs(got - want).max() <= own + bound(want), (kind, mode, loop, sweeps)
                assert res["refinements"] >= 1 and res["last_delta"] < 1e-10
                assert res["affected_initial"] == r64["affected_initial"]
    finally:
        g.close()


def test_refine_dynamic_caps_and_empty_batch(pg, ctx):
    xoff, xedg = pg.graphs.rmat(12, 16, seed=5)
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, 20, 80, seed=31)
    du, dv, iu, iv = batch
    xt = O.transpose(xoff, xedg)
    q, _ = O.solve("static", None, None, *xt)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    g = pg.Graph(ctx, *yt, yoff, yedg)
    try:
        for sweeps in (1, 2):
            for L in (0, 1, 3):
                got, res = pg.solve(ctx, g, pg.PRUNE_DYNAMIC_FRONTIER, (du, dv), (iu, iv), q,
                                    pg.options(precision=pg.FP32_REFINE, max_iterations=L, refine_sweeps=sweeps))
                assert res["iterations"] == L and np.all(np.isfinite(got)), (sweeps, L)
                if L == 0:
                    np.testing.assert_array_equal(got, q)
        e = np.zeros(0, np.uint32)
        want, _ = O.solve("prune_dynamic_frontier", yoff, yedg, *yt, e, e, e, e, q=q)
        got, res = pg.solve(ctx, g, pg.PRUNE_DYNAMIC_FRONTIER, (e, e), (e, e), q,
                            pg.options(precision=pg.FP32_REFINE))
        assert res["affected_initial"] == 0
        conv, _ = O.solve("static", None, None, *yt)
        assert np.abs(got - conv).max() <= bound(conv)
        assert np.abs(got - want).max() <= np.abs(want - conv).max() + bound(want)
    finally:
        g.close()


@pytest.mark.parametrize("kind", ["web200k", "hubs"])
def test_refine_graph_and_host_loops_agree(pg, ctx, kind):
    # The refinement's rounds run as one CUDA graph launch (outer WHILE node of
    # FP64 residual sweeps, inner WHILE node of FP32 sweeps) or from the host:
    # the same sweeps in the same order, so the same bits, iterations and
    # refinement rounds, also when the iteration cap ends an FP32 round
    from test_gpu_parity import _synthetic
    xoff, xedg = _synthetic(pg, kind)
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, max(1, int(2e-4 * m)), max(1, int(8e-4 * m)), seed=37)
    du, dv, iu, iv = batch
    q, _ = pg.pagerank_static(ctx, pg.Graph.from_out_csr(ctx, xoff, xedg))
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    g = pg.Graph(ctx, *yt, yoff, yedg)
    try:
        cases = [(pg.STATIC, None, 0), (pg.NAIVE_DYNAMIC, None, 0)]
        cases += [(mode, batch, sweeps) for mode in (pg.DYNAMIC_FRONTIER, pg.PRUNE_DYNAMIC_FRONTIER)
                  for sweeps in (1, 2)]
        for mode, b, sweeps in cases:
            for cap in (500, 3, 6, 9):
                out = []
                for loop in (pg.LOOP_GRAPH, pg.LOOP_HOST):
                    o = pg.options(precision=pg.FP32_REFINE, loop=loop, refine_sweeps=sweeps, max_iterations=cap)
                    if b is None:
                        out.append(pg.solve(ctx, g, mode, q=q if mode != pg.STATIC else None, opts=o))
                    else:
                        out.append(pg.solve(ctx, g, mode, (du, dv), (iu, iv), q, o))
                (a, ra), (h, rh) = out
                assert np.array_equal(a, h), (kind, mode, sweeps, cap)
                assert ra["iterations"] == rh["iterations"] and ra["refinements"] == rh["refinements"]
                assert ra["last_delta"] == rh["last_delta"]
    finally:
        g.close()
