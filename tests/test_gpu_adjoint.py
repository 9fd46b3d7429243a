"""Weighted PageRank and its adjoint on the GPU against the dense FP64
oracle (oracle/adjoint_oracle.py) and central finite differences of GPU
forward solves.  No counterpart in the reference (unweighted graphs only)."""
import numpy as np
import pytest

from oracle import adjoint_oracle as AO
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    return pagerank_gb300


@pytest.fixture(scope="module")
def A():
    from pagerank_gb300 import autograd
    return autograd


def _weighted(pg, A, ctx, scale, seed):
    import torch
    xoff, xedg = pg.graphs.rmat(scale, 16, seed=seed)
    xt = O.transpose(xoff, xedg)
    g = pg.Graph(ctx, *xt, xoff, xedg)
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.5, 2.0, len(xedg)).astype(np.float32)
    A.set_weights(ctx, g, torch.from_numpy(w).cuda())
    return g, xoff, xedg, w, rng


def test_adjoint_matches_dense_solve(pg, A, ctx):
    import torch
    g, xoff, xedg, w, rng = _weighted(pg, A, ctx, 10, 4)
    n = len(xoff) - 1
    t = rng.dirichlet(np.ones(n))
    gl = rng.standard_normal(n)
    a = 0.85
    r_want, lam_want, gw_want, gt_want, ga_want = AO.gradients(xoff, xedg, w.astype(np.float64), t, a, gl)
    o = pg.options(damping=a, tolerance=1e-15, max_iterations=3000)
    tt = torch.from_numpy(t).cuda()
    r, res = A.solve_weighted(ctx, g, tt, opts=o)
    assert np.abs(r.cpu().numpy() - r_want).max() <= 1e-13
    out = A.adjoint(ctx, g, r, torch.from_numpy(gl).cuda(), tt, opts=o, want_lambda=True)
    assert np.abs(out["lambda"].cpu().numpy() - lam_want).max() <= 1e-11 * np.abs(lam_want).max()
    gw = out["grad_w"].cpu().numpy()
    assert np.abs(gw - gw_want).max() <= 1e-9 * np.abs(gw_want).max()
    assert np.abs(out["grad_t"].cpu().numpy() - gt_want).max() <= 1e-9 * np.abs(gt_want).max()
    assert abs(out["grad_alpha"] - ga_want) <= 1e-9 * abs(ga_want)
    # uniform teleport (t = NULL) equals an explicit uniform vector
    ru, _ = A.solve_weighted(ctx, g, None, opts=o)
    r1, _ = A.solve_weighted(ctx, g, torch.full((n,), 1.0 / n, dtype=torch.float64, device="cuda"), opts=o)
    assert torch.equal(ru, r1)
    g.close()


def test_adjoint_matches_gpu_finite_differences(pg, A, ctx):
    # dL/dw of L = g . r by central differences (h = 1e-6) of GPU forward
    # solves, the differences formed without cancellation: 1e-6 relative.
    import torch
    g, xoff, xedg, w, rng = _weighted(pg, A, ctx, 12, 8)
    n, m = len(xoff) - 1, len(xedg)
    gl = torch.from_numpy(rng.standard_normal(n)).cuda()
    o = pg.options(tolerance=1e-19, max_iterations=2000)
    r, _ = A.solve_weighted(ctx, g, None, opts=o)
    adj = A.adjoint(ctx, g, r, gl, None, opts=o)["grad_w"].cpu().numpy()
    edges = rng.choice(m, 24, replace=False)
    fd = A.fd_weight_gradients(ctx, g, xoff, xedg, w, r, gl, edges)
    assert np.abs(fd - adj[edges]).max() <= 1e-6 * np.abs(adj[edges]).max()
    g.close()


def test_autograd_function(pg, A, ctx):
    import torch
    g, xoff, xedg, w, rng = _weighted(pg, A, ctx, 11, 6)
    n = len(xoff) - 1
    wt = torch.from_numpy(w).cuda().requires_grad_(True)
    t = torch.from_numpy(rng.dirichlet(np.ones(n))).cuda().requires_grad_(True)
    alpha = torch.tensor(0.8, dtype=torch.float64, device="cuda", requires_grad=True)
    gv = torch.from_numpy(rng.standard_normal(n)).cuda()
    r = A.weighted_pagerank(ctx, g, wt, t, alpha, tolerance=1e-14)
    (gv * r).sum().backward()
    o = pg.options(damping=0.8, tolerance=1e-14, max_iterations=1000)
    A.set_weights(ctx, g, wt)
    r2, _ = A.solve_weighted(ctx, g, t.detach(), opts=o)
    assert torch.equal(r.detach(), r2)
    out = A.adjoint(ctx, g, r2, gv, t.detach(), opts=o)
    assert torch.equal(wt.grad, out["grad_w"].to(torch.float32))
    assert torch.equal(t.grad, out["grad_t"])
    assert alpha.grad.item() == out["grad_alpha"]
    g.close()


def test_weights_lifecycle_and_errors(pg, A, ctx):
    import torch
    g, xoff, xedg, w, rng = _weighted(pg, A, ctx, 9, 2)
    batch = pg.graphs.random_batch(xoff, xedg, 5, 20, seed=3)
    g.apply_batch(*batch)                      # edges changed: weights dropped
    with pytest.raises(pg.PrxError) as e:
        A.solve_weighted(ctx, g)
    assert e.value.status == 6
    _, m2 = g.size()
    A.set_weights(ctx, g, torch.ones(m2, dtype=torch.float32, device="cuda"))
    r, res = A.solve_weighted(ctx, g, opts=pg.options(tolerance=1e-12))
    assert res["iterations"] > 0 and abs(float(r.sum()) - 1) < 1e-9
    bad = torch.ones(m2, dtype=torch.float32, device="cuda")
    bad[7] = 0.0
    with pytest.raises(pg.PrxError) as e:
        A.set_weights(ctx, g, bad)
    assert e.value.status == 1
    with pytest.raises(pg.PrxError) as e:          # the failed call left no weights
        A.solve_weighted(ctx, g)
    assert e.value.status == 6
    xt = O.transpose(xoff, xedg)
    g2 = pg.Graph(ctx, *xt)                         # no out-CSR
    with pytest.raises(pg.PrxError) as e:
        A.set_weights(ctx, g2, torch.ones(len(xedg), dtype=torch.float32, device="cuda"))
    assert e.value.status == 6
    g2.close()
    g.close()
