"""The dense adjoint oracle's gradient formulas against central finite
differences of the same dense solves (CPU; pins the mathematics that the
GPU adjoint is checked against)."""
import numpy as np

from oracle import adjoint_oracle as AO


def _graph(n=200, deg=6, seed=1):
    rng = np.random.default_rng(seed)
    rows = []
    for u in range(n):
        nb = set(rng.integers(0, n, deg).tolist()) | {u}   # self-loop: no dangling vertex
        rows.append(sorted(nb))
    off = np.zeros(n + 1, np.int64)
    off[1:] = np.cumsum([len(r) for r in rows])
    edg = np.concatenate([np.array(r) for r in rows])
    return off, edg, rng


def test_adjoint_formulas_match_finite_differences():
    off, edg, rng = _graph()
    n, m = len(off) - 1, len(edg)
    w = rng.uniform(0.5, 2.0, m)
    t = rng.dirichlet(np.ones(n))
    g = rng.standard_normal(n)
    a = 0.85
    r, lam, gw, gt, ga = AO.gradients(off, edg, w, t, a, g)
    assert abs(r.sum() - 1) < 1e-12
    edges = rng.choice(m, 40, replace=False)
    fd = AO.fd_weights(off, edg, w, t, a, g, edges)
    assert np.abs(fd - gw[edges]).max() <= 1e-6 * np.abs(gw[edges]).max()
    verts = rng.choice(n, 10, replace=False)
    fdt = AO.fd_teleport(off, edg, w, t, a, g, verts)
    assert np.abs(fdt - gt[verts]).max() <= 1e-6 * np.abs(gt[verts]).max()
    assert abs(AO.fd_alpha(off, edg, w, t, a, g) - ga) <= 1e-6 * abs(ga)
