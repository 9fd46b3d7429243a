"""FP64 oracle of the batched personalized PageRank (test infrastructure only).

Batched personalized PageRank has no counterpart in the reference (whose
solvers use the uniform teleport (1-P)/N only, inc/pagerankCuda.hxx:679), so
this oracle is the mathematics itself, in numpy / scipy:

    r_k = (1 - P) t_k + P * A^T D^-1 r_k,   t_k = (1/|S_k|) sum_{s in S_k} e_s,

iterated by Jacobi sweeps from r_k = t_k until the L-inf change of one sweep
over all vertices and the vectors of a block of 64 is below the tolerance
(the reference's stopping rule, inc/pagerankCuda.hxx:680,689, applied per
block of 64 vectors as the library does), and the same sweeps run to the
FP64 floor for the converged answer.  Parity is therefore pinned to
the definition, not to reference outputs.
"""
import numpy as np
import scipy.sparse as sp

BLOCK = 64


def teleport(n, seed_sets):
    """Dense t [n, nvec]: 1/|S_k| per occurrence of a seed in S_k."""
    t = np.zeros((n, len(seed_sets)))
    for k, s in enumerate(seed_sets):
        s = np.asarray(s, dtype=np.int64)
        np.add.at(t[:, k], s, 1.0 / len(s))
    return t


def _operator(xtoff, xtedg, xtdat):
    n = len(xtoff) - 1
    a = sp.csr_matrix((np.ones(len(xtedg)), np.asarray(xtedg, np.int64), np.asarray(xtoff, np.int64)), shape=(n, n))
    d = np.asarray(xtdat, np.float64)
    dinv = np.divide(1.0, d, out=np.zeros_like(d), where=d > 0)
    return a, dinv


def jacobi(xtoff, xtedg, xtdat, seed_sets, damping=0.85, tol=1e-10, max_iter=500):
    """Jacobi sweeps per block of 64 vectors -> (ranks [n, nvec], sweeps per block)."""
    n = len(xtoff) - 1
    a, dinv = _operator(xtoff, xtedg, xtdat)
    t = teleport(n, seed_sets)
    out = np.zeros_like(t)
    iters = []
    for c0 in range(0, t.shape[1], BLOCK):
        tb = t[:, c0:c0 + BLOCK]
        r = tb.copy()
        it = 0
        while it < max_iter:
            nr = (1 - damping) * tb + damping * (a @ (r * dinv[:, None]))
            delta = np.abs(nr - r).max()
            r = nr
            it += 1
            if delta < tol:
                break
        out[:, c0:c0 + BLOCK] = r
        iters.append(it)
    return out, iters


def exact(xtoff, xtedg, xtdat, seed_sets, damping=0.85):
    """The converged answer: Jacobi sweeps to an L-inf change of 1e-15 (the
    FP64 floor for ranks <= 1), or 5000 sweeps."""
    r, _ = jacobi(xtoff, xtedg, xtdat, seed_sets, damping=damping, tol=1e-15, max_iter=5000)
    return r
