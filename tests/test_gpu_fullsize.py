"""Full-size parity on the benchmark graphs, through the C ABI.

* The 4096 x 4096 road-like grid (16.8M vertices, 85.5M edges: 4-neighbour
  edges both ways, 5% diagonal shortcuts, self-loops): Static FP64 and, after
  one batch of 1e-4 |E| (80% insertions) applied on the device, DT, DF and
  DF-P -- ranks bit-identical to the oracle's restatement of the reference's
  GPU solvers (inc/pagerankCuda.hxx:675-692) with equal iteration counts.
* The web-like graph (50M vertices, 1.9B edges, Zipf(2.1) out-degree, 70% of
  targets within +/-4096 ids): Static FP64 bit-identical to the same
  restatement with equal iterations, and within L-inf 1e-9 of the
  reference's OpenMP Static (pagerankStaticOmp, inc/pagerank.hxx:474-482)
  with equal iterations; DF and DF-P after the first 1e-4 |E| batch
  bit-identical to the restatement.

The oracle runs its sweeps with OpenMP threads (vertices are independent
within a sweep, so the threads change no bit).  Host memory: about 45 GB for
the web-like graph's arrays; device memory: about 20 GB."""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    return pagerank_gb300


def _batch(pg, xoff, xedg, frac, seed):
    m = len(xedg)
    size = int(frac * m)
    return pg.graphs.random_batch(xoff, xedg, size // 5, size - size // 5, seed=seed)


def _check(pg, ctx, g, mode, yoff, yedg, yt, batch, q):
    du, dv, iu, iv = batch
    want, it = O.solve(mode, yoff, yedg, *yt, du, dv, iu, iv, q=q)
    got, res = pg.solve(ctx, g, pg.MODES[mode], (du, dv), (iu, iv), q)
    assert res["iterations"] == it, (mode, res["iterations"], it)
    assert np.array_equal(got, want), (mode, float(np.abs(got - want).max()))
    return got


def test_grid4096_static_and_dynamic_bit_exact(pg, ctx):
    xoff, xedg = pg.graphs.grid(4096, 0.05, seed=42)
    xt = O.transpose(xoff, xedg, threads=True)
    n, m = len(xoff) - 1, len(xedg)
    assert n == 4096 * 4096 and m > 80_000_000
    g = pg.Graph(ctx, *xt, xoff, xedg)
    try:
        want, it = O.solve("static", None, None, *xt)
        got, res = pg.pagerank_static(ctx, g)
        assert res["iterations"] == it
        assert np.array_equal(got, want)
        batch = _batch(pg, xoff, xedg, 1e-4, seed=45)
        yoff, yedg = O.apply_batch(xoff, xedg, *batch)
        yt = O.transpose(yoff, yedg, threads=True)
        g.apply_batch(*batch)
        for mode in ("dynamic_traversal", "dynamic_frontier", "prune_dynamic_frontier"):
            _check(pg, ctx, g, mode, yoff, yedg, yt, batch, want)
    finally:
        g.close()


def test_weblike50m_static_and_dynamic_bit_exact(pg, ctx):
    xoff, xedg = pg.graphs.weblike(50_000_000, alpha=2.1, dmin=5.9, dmax=100000, local=0.7, window=4096, seed=42)
    xt = O.transpose(xoff, xedg, threads=True)
    m = len(xedg)
    assert m > 1_800_000_000
    g = pg.Graph(ctx, *xt, xoff, xedg)
    try:
        want, it = O.solve("static", None, None, *xt)
        got, res = pg.pagerank_static(ctx, g)
        assert res["iterations"] == it
        assert np.array_equal(got, want)
        cpu, it_cpu = O.cpu_static(*xt)
        assert it_cpu == it
        assert float(np.abs(got - cpu).max()) <= 1e-9
        del cpu
        batch = _batch(pg, xoff, xedg, 1e-4, seed=43)
        yoff, yedg = O.apply_batch(xoff, xedg, *batch)
        del xt, xoff, xedg
        yt = O.transpose(yoff, yedg, threads=True)
        g.apply_batch(*batch)
        for mode in ("dynamic_frontier", "prune_dynamic_frontier"):
            _check(pg, ctx, g, mode, yoff, yedg, yt, batch, want)
    finally:
        g.close()
