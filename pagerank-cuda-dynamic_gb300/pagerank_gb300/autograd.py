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


__all__ = ["set_weights", "solve_weighted", "adjoint", "WeightedPageRank", "weighted_pagerank"]
