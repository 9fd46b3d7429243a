"""Weighted PageRank as a differentiable torch op over the C ABI.

prx_solve_weighted gives the ranks r = (1 - alpha) t + alpha P^T r of a
graph whose edge weights are row-normalised (P_uv = w_uv / W_u);
prx_adjoint solves lambda = alpha P lambda + dL/dr with the same pull kernels
on the reversed graph and returns dL/dw, dL/dt and dL/dalpha.  Only the
converged ranks are kept for the backward pass, not per-iteration state.

The library runs on its context's own stream and returns after its work
finished; the calls here first wait for torch's current stream so that the
tensors they read are ready.
"""
import ctypes as C

import torch

from ._lib import Result, check, load
from .api import options


def _ptr(x):
    return None if x is None else x.data_ptr()


def _f64(x):
    return x.detach().to(dtype=torch.float64).contiguous()


def set_weights(ctx, g, weights):
    """Attach edge weights (m values in out-CSR order, device tensor)."""
    w = weights.detach().to(device="cuda", dtype=torch.float32).contiguous()
    torch.cuda.current_stream().synchronize()
    check(load().prx_graph_set_weights(ctx.handle, g.handle, w.data_ptr()), "prx_graph_set_weights")


def solve_weighted(ctx, g, teleport=None, r0=None, opts=None):
    """Converged ranks (float64 device tensor) and the result dict."""
    n, _ = g.size()
    t = None if teleport is None else _f64(teleport)
    s0 = None if r0 is None else _f64(r0)
    r = torch.empty(n, dtype=torch.float64, device="cuda")
    res = Result()
    torch.cuda.current_stream().synchronize()
    check(load().prx_solve_weighted(ctx.handle, g.handle, _ptr(t), _ptr(s0), C.byref(opts or options()),
                                    r.data_ptr(), C.byref(res)), "prx_solve_weighted")
    return r, res.as_dict()


def adjoint(ctx, g, r, grad_r, teleport=None, opts=None, want_lambda=False):
    """-> dict(grad_w (m), grad_t (n), grad_alpha (float), lambda (n, optional), result)."""
    n, m = g.size()
    t = None if teleport is None else _f64(teleport)
    rr, gl = _f64(r), _f64(grad_r)
    gw = torch.empty(m, dtype=torch.float64, device="cuda")
    gt = torch.empty(n, dtype=torch.float64, device="cuda")
    lam = torch.empty(n, dtype=torch.float64, device="cuda") if want_lambda else None
    ga = C.c_double(0.0)
    res = Result()
    torch.cuda.current_stream().synchronize()
    check(load().prx_adjoint(ctx.handle, g.handle, _ptr(t), rr.data_ptr(), gl.data_ptr(), C.byref(opts or options()),
                             _ptr(lam), gw.data_ptr(), gt.data_ptr(), C.byref(ga), C.byref(res)), "prx_adjoint")
    out = {"grad_w": gw, "grad_t": gt, "grad_alpha": ga.value, "result": res.as_dict()}
    if want_lambda:
        out["lambda"] = lam
    return out


def fd_weight_gradients(ctx, g, xoff, xedg, weights, r, grad_r, edges, h=1e-6, teleport=None, alpha=0.85,
                        tolerance=1e-24, max_iterations=3000):
    """Central finite differences of L = grad_r . r with respect to the weights
    of the given out-CSR edges: (L(w + h e_j) - L(w - h e_j)) / (w+_j - w-_j),
    with w+-_j rounded to FP32 as the library stores them.

    The two differences L(w +- h e_j) - L(w) are formed without cancellation:
    r+- - r solves (I - alpha P+-^T) d = alpha (P+- - P)^T r exactly, a system
    whose right-hand side is non-zero only on the out-neighbours of the edge's
    source, solved by the library's weighted solver with that right-hand side
    as (1 - alpha) times its teleport vector.  r must be the converged ranks
    for `weights` (tightly converged: its residual enters both differences).
    Leaves `weights` attached to g.  Returns a float64 numpy array."""
    import numpy as np
    xoff = np.asarray(xoff, np.int64)
    w = np.asarray(weights.detach().cpu().numpy() if isinstance(weights, torch.Tensor) else weights, np.float32)
    dev = r.device
    gl = _f64(grad_r)
    n = len(xoff) - 1
    o = options(damping=alpha, tolerance=tolerance, max_iterations=max_iterations)
    wd = torch.from_numpy(w).to(dev)   # one device copy; each difference changes one entry in place
    rh = r.detach().cpu().numpy() if isinstance(r, torch.Tensor) else np.asarray(r)
    out = []
    for j in edges:
        u = int(np.searchsorted(xoff, j, side="right") - 1)
        s, e = xoff[u], xoff[u + 1]
        nb = torch.from_numpy(np.asarray(xedg[s:e], np.int64)).to(dev)
        row = w[s:e].astype(np.float64)
        ru = float(rh[u])
        diffs = []
        wj = []
        for sign in (1.0, -1.0):
            wq_j = np.float32(w[j] + np.float32(sign * h))
            wj.append(float(wq_j))
            rq = row.copy()
            rq[j - s] = float(wq_j)
            b = alpha * ru * (rq / rq.sum() - row / row.sum())     # alpha (Pq - P)^T r, rows of u only
            t = torch.zeros(n, dtype=torch.float64, device=dev)
            t.index_add_(0, nb, torch.from_numpy(b / (1 - alpha)).to(dev))
            wd[j] = float(wq_j)
            set_weights(ctx, g, wd)
            d, _ = solve_weighted(ctx, g, t, opts=o)
            diffs.append(float((gl * d).sum()))
        wd[j] = float(w[j])
        out.append((diffs[0] - diffs[1]) / (wj[0] - wj[1]))
    set_weights(ctx, g, wd)
    return np.array(out)


class WeightedPageRank(torch.autograd.Function):
    """r = WeightedPageRank.apply(weights, teleport, alpha, ctx, graph, tolerance, max_iterations).

    weights: (m,) edge weights in out-CSR order; teleport: (n,) or None
    (uniform); alpha: float or 0-d tensor.  Gradients flow to all three."""

    @staticmethod
    def forward(fctx, weights, teleport, alpha, pctx, graph, tolerance, max_iterations):
        a = float(alpha)
        o = options(damping=a, tolerance=tolerance, max_iterations=max_iterations)
        set_weights(pctx, graph, weights)
        r, _ = solve_weighted(pctx, graph, teleport, opts=o)
        fctx.pctx, fctx.graph, fctx.opts = pctx, graph, o
        fctx.teleport_given = teleport is not None
        fctx.alpha_tensor = isinstance(alpha, torch.Tensor)
        fctx.save_for_backward(weights, teleport if teleport is not None else torch.empty(0), r)
        return r

    @staticmethod
    def backward(fctx, grad_r):
        weights, teleport, r = fctx.saved_tensors
        t = teleport if fctx.teleport_given else None
        set_weights(fctx.pctx, fctx.graph, weights)  # the graph may have been given other weights since
        out = adjoint(fctx.pctx, fctx.graph, r, grad_r, t, fctx.opts)
        gw = out["grad_w"].to(weights.dtype) if fctx.needs_input_grad[0] else None
        gt = out["grad_t"].to(teleport.dtype) if fctx.teleport_given and fctx.needs_input_grad[1] else None
        ga = None
        if fctx.alpha_tensor and fctx.needs_input_grad[2]:
            ga = torch.tensor(out["grad_alpha"], dtype=torch.float64, device=r.device)
        return gw, gt, ga, None, None, None, None


def weighted_pagerank(pctx, graph, weights, teleport=None, alpha=0.85, tolerance=1e-12, max_iterations=1000):
    """Differentiable weighted PageRank (see WeightedPageRank)."""
    return WeightedPageRank.apply(weights, teleport, alpha, pctx, graph, tolerance, max_iterations)


__all__ = ["set_weights", "solve_weighted", "adjoint", "fd_weight_gradients", "WeightedPageRank",
           "weighted_pagerank"]
