"""Batched personalized PageRank on the GPU against its FP64 oracle.

The solver has no counterpart in the reference, so the oracle is the
definition (oracle/ppr_oracle.py): Jacobi sweeps in numpy with the same
stopping rule, and a direct sparse solve.  Sums run in another order on the
GPU, so ranks agree to rounding (1e-12) rather than bit for bit; the
FP32-refined path must be about as close to the converged answer as FP64
Jacobi stopped by the same tolerance."""
import numpy as np
import pytest

from oracle import ppr_oracle as PO
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    return pagerank_gb300


def _graph(pg, ctx, kind):
    if kind == "rmat12":
        xoff, xedg = pg.graphs.rmat(12, 16, seed=5)
    elif kind == "hubs":      # in-degrees up to thousands: several 512-edge segments per row
        xoff, xedg = pg.graphs.rmat(14, 48, a=0.7, b=0.1, c=0.1, seed=3)
    elif kind == "web20k":
        xoff, xedg = pg.graphs.weblike(20000, dmax=2000, window=1024, seed=9)
    else:
        raise KeyError(kind)
    xt = O.transpose(xoff, xedg)
    return pg.Graph(ctx, *xt), xt


def _seeds(n, nvec, seed):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(0, np.log(50), nvec)).astype(int) + 1  # log-uniform in [1, 50]
    return [rng.integers(0, n, s) for s in sizes]


@pytest.mark.parametrize("kind,nvec", [("rmat12", 64), ("hubs", 16), ("web20k", 70)])
def test_ppr_fp64_matches_jacobi(pg, ctx, kind, nvec):
    g, xt = _graph(pg, ctx, kind)
    n = len(xt[0]) - 1
    seeds = _seeds(n, nvec, 17)
    want, its = PO.jacobi(*xt, seeds, tol=1e-10)
    got, res = pg.solve_ppr_batched(ctx, g, seeds, pg.options(tolerance=1e-10))
    assert got.shape == (n, nvec)
    assert res["iterations"] == max(its)
    assert res["fp64_sweeps"] == sum(its)
    assert np.abs(got - want).max() <= 1e-12
    # every column is a probability distribution (self-loops: no dangling mass)
    np.testing.assert_allclose(got.sum(axis=0), 1.0, atol=1e-8)
    g.close()


@pytest.mark.parametrize("kind,nvec", [("rmat12", 64), ("hubs", 33), ("web20k", 64)])
def test_ppr_fp32_refine_accuracy(pg, ctx, kind, nvec):
    g, xt = _graph(pg, ctx, kind)
    n = len(xt[0]) - 1
    seeds = _seeds(n, nvec, 23)
    exact = PO.exact(*xt, seeds)
    tol = 1e-10
    got, res = pg.solve_ppr_batched(ctx, g, seeds, pg.options(tolerance=tol, precision=pg.FP32_REFINE))
    ref64, _ = pg.solve_ppr_batched(ctx, g, seeds, pg.options(tolerance=tol))
    err64 = np.abs(ref64 - exact).max()
    assert err64 <= 100 * tol
    assert np.abs(got - exact).max() <= max(2 * err64, tol)
    assert res["fp32_sweeps"] > 0 and res["refinements"] >= 2
    assert res["last_delta"] < tol
    g.close()


def test_ppr_deterministic_and_device_output(pg, ctx):
    import torch
    g, xt = _graph(pg, ctx, "hubs")
    n = len(xt[0]) - 1
    seeds = _seeds(n, 40, 31)
    for prec in (pg.FP64, pg.FP32_REFINE):
        o = pg.options(tolerance=1e-9, precision=prec)
        a, _ = pg.solve_ppr_batched(ctx, g, seeds, o)
        b, _ = pg.solve_ppr_batched(ctx, g, seeds, o)
        np.testing.assert_array_equal(a, b)
        out = torch.empty(n * 40, dtype=torch.float64, device="cuda")
        pg.solve_ppr_batched_device(ctx, g, seeds, out.data_ptr(), o)
        np.testing.assert_array_equal(out.cpu().numpy().reshape(n, 40), a)
    g.close()


def test_ppr_caps_and_errors(pg, ctx):
    g, xt = _graph(pg, ctx, "rmat12")
    n = len(xt[0]) - 1
    seeds = [[0], [1, 1, 2]]                       # a repeated seed counts twice
    r, res = pg.solve_ppr_batched(ctx, g, seeds, pg.options(max_iterations=0))
    t = PO.teleport(n, seeds)
    np.testing.assert_array_equal(r, t)
    assert res["iterations"] == 0
    want, _ = PO.jacobi(*xt, seeds, max_iter=3)
    r, res = pg.solve_ppr_batched(ctx, g, seeds, pg.options(max_iterations=3))
    assert res["iterations"] == 3 and np.abs(r - want).max() <= 1e-14
    for prec in (pg.FP64, pg.FP32_REFINE):
        r, res = pg.solve_ppr_batched(ctx, g, seeds, pg.options(max_iterations=5, precision=prec))
        assert res["iterations"] == 5
    with pytest.raises(pg.PrxError) as e:
        pg.solve_ppr_batched(ctx, g, [[0], []])
    assert e.value.status == 1
    with pytest.raises(pg.PrxError) as e:
        pg.solve_ppr_batched(ctx, g, [[n]])
    assert e.value.status == 1
    with pytest.raises(pg.PrxError) as e:
        pg.solve_ppr_batched(ctx, g, [])
    assert e.value.status == 1
    g.close()


@pytest.mark.parametrize("kind,nvec", [("rmat12", 64), ("hubs", 70), ("web20k", 33)])
def test_ppr_graph_loop_equals_host_loop(pg, ctx, kind, nvec):
    # the iteration loop of a block as one CUDA graph launch (a WHILE node,
    # and for the refinement a nested WHILE node over each round's FP32
    # sweeps) runs the host loop's kernels in the same order: bit-identical
    # ranks and equal sweep counts, also when the iteration cap stops a round
    g, xt = _graph(pg, ctx, kind)
    n = len(xt[0]) - 1
    seeds = _seeds(n, nvec, 41)
    blocks = (nvec + 63) // 64
    for prec in (pg.FP64, pg.FP32_REFINE):
        for cap in (500, 1, 2, 7):
            kw = dict(tolerance=1e-10, precision=prec, max_iterations=cap)
            host, rh = pg.solve_ppr_batched(ctx, g, seeds, pg.options(loop=pg.LOOP_HOST, **kw))
            got, rg = pg.solve_ppr_batched(ctx, g, seeds, pg.options(**kw))
            np.testing.assert_array_equal(got, host, err_msg=f"{kind} prec={prec} cap={cap}")
            for k in ("iterations", "fp64_sweeps", "fp32_sweeps", "refinements"):
                assert rg[k] == rh[k], (k, kind, prec, cap)
            assert rg["graph_launches"] == blocks and rh["graph_launches"] == 0
    g.close()


@pytest.mark.parametrize("kind", ["hubs", "web20k"])
def test_ppr_autotuned_split(pg, ctx, kind):
    # prx_autotune_ppr keeps a (warp-per-vertex bound, segment width) pair on
    # the graph; every split gives the oracle's answer to rounding
    g, xt = _graph(pg, ctx, kind)
    n = len(xt[0]) - 1
    seeds = _seeds(n, 20, 43)
    want, its = PO.jacobi(*xt, seeds, tol=1e-10)
    pick = pg.autotune_ppr(ctx, g)
    assert pick["low_max"] in (64, 256, 1024) and pick["seg_edges"] in (256, 512, 1024, 2048)
    assert pick["trials"] == 12
    got, res = pg.solve_ppr_batched(ctx, g, seeds, pg.options(tolerance=1e-10))
    assert (res["low_max"], res["seg_edges"]) == (pick["low_max"], pick["seg_edges"])
    assert res["iterations"] == max(its)
    assert np.abs(got - want).max() <= 1e-12
    g.close()
