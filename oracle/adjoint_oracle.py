"""Dense FP64 oracle of weighted PageRank and its adjoint (test infrastructure only).

Weighted PageRank and its adjoint have no counterpart in the reference (its
graphs are unweighted, inc/pagerankCuda.hxx:87-109), so this oracle is the
mathematics, in dense numpy:

    P_uv = w_uv / W_u,   r = (1 - a) t + a P^T r,   L = g . r,
    lambda = a P lambda + g,
    dL/dw_uv = (r_u / W_u)(a lambda_v - lambda_u + g_u),
    dL/dt = (1 - a) lambda,   dL/da = lambda . (P^T r - t),

with direct solves of the two linear systems, and central finite differences
of L through the same direct solves to pin those gradient formulas.
"""
import numpy as np


def dense_p(xoff, xedg, w):
    n = len(xoff) - 1
    p = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(np.asarray(xoff, np.int64)))
    w = np.asarray(w, np.float64)
    ws = np.bincount(rows, weights=w, minlength=n)
    p[rows, np.asarray(xedg, np.int64)] = w / ws[rows]
    return p, ws


def ranks(p, t, a):
    n = p.shape[0]
    return np.linalg.solve(np.eye(n) - a * p.T, (1 - a) * t)


def adjoint(p, g, a):
    n = p.shape[0]
    return np.linalg.solve(np.eye(n) - a * p, g)


def gradients(xoff, xedg, w, t, a, g):
    """-> r, lambda, dL/dw (out-CSR order), dL/dt, dL/da."""
    p, ws = dense_p(xoff, xedg, w)
    r = ranks(p, t, a)
    lam = adjoint(p, g, a)
    n = len(xoff) - 1
    rows = np.repeat(np.arange(n), np.diff(np.asarray(xoff, np.int64)))
    cols = np.asarray(xedg, np.int64)
    gw = (r[rows] / ws[rows]) * (a * lam[cols] - lam[rows] + g[rows])
    gt = (1 - a) * lam
    ga = lam @ (p.T @ r - t)
    return r, lam, gw, gt, ga


def loss(xoff, xedg, w, t, a, g):
    p, _ = dense_p(xoff, xedg, w)
    return g @ ranks(p, t, a)


def fd_weights(xoff, xedg, w, t, a, g, edges, h=1e-6):
    w = np.asarray(w, np.float64)
    out = []
    for j in edges:
        wp, wm = w.copy(), w.copy()
        wp[j] += h
        wm[j] -= h
        out.append((loss(xoff, xedg, wp, t, a, g) - loss(xoff, xedg, wm, t, a, g)) / (2 * h))
    return np.array(out)


def fd_alpha(xoff, xedg, w, t, a, g, h=1e-6):
    return (loss(xoff, xedg, w, t, a + h, g) - loss(xoff, xedg, w, t, a - h, g)) / (2 * h)


def fd_teleport(xoff, xedg, w, t, a, g, verts, h=1e-6):
    out = []
    for v in verts:
        tp, tm = t.copy(), t.copy()
        tp[v] += h
        tm[v] -= h
        out.append((loss(xoff, xedg, w, tp, a, g) - loss(xoff, xedg, w, tm, a, g)) / (2 * h))
    return np.array(out)
