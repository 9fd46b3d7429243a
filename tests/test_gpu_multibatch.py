"""prx_solve_batches_device: K consecutive batches applied and solved in one
CUDA graph launch must give, batch after batch, the bits of the host loop
the reference's driver runs (main.cu:88-147): apply batch k, then solve from
the previous batch's ranks."""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    pagerank_gb300.load()
    return pagerank_gb300


def _graph(pg, kind):
    if kind == "rmat":
        return pg.graphs.rmat(14, 12, seed=6)
    if kind == "web":
        return pg.graphs.weblike(120_000, seed=6)
    return pg.graphs.grid(160, seed=6)


def _batches(pg, xoff, xedg, K, seed):
    """K batches, each tidy against the graph the ones before it leave."""
    out = []
    for k in range(K):
        m = len(xedg)
        size = max(8, int(2e-3 * m) * (k + 1))
        b = pg.graphs.random_batch(xoff, xedg, size // 4, size - size // 4, seed=seed + k)
        out.append(b)
        xoff, xedg = pg.graphs.apply_batch(xoff, xedg, *b)
    return out


@pytest.mark.parametrize("kind", ["rmat", "web", "grid"])
@pytest.mark.parametrize("mode", ["dynamic_frontier", "prune_dynamic_frontier"])
def test_batches_in_one_launch_equal_host_loop(pg, ctx, kind, mode):
    xoff, xedg = _graph(pg, kind)
    batches = _batches(pg, xoff, xedg, 4, seed=20)
    xt = O.transpose(xoff, xedg)
    ref = pg.Graph(ctx, *xt, xoff, xedg)
    q0, _ = pg.pagerank_static(ctx, ref)
    want, want_res, q = [], [], q0
    for b in batches:
        ref.apply_batch(*b)
        q, r = pg.solve(ctx, ref, pg.MODES[mode], b[:2], b[2:], q)
        want.append(q)
        want_res.append(r)
    mb = pg.Graph(ctx, *xt, xoff, xedg)
    last, res, each = pg.solve_batches(ctx, mb, pg.MODES[mode], batches, q0, each=True)
    assert len(res) == len(batches)
    for k in range(len(batches)):
        assert res[k]["iterations"] == want_res[k]["iterations"], (kind, mode, k)
        assert res[k]["affected_initial"] == want_res[k]["affected_initial"]
        assert np.array_equal(each[k], want[k]), (kind, mode, k)
    assert np.array_equal(last, want[-1])
    # the graph is left at the last version, and solves on it as usual
    a, b = ref.download(), mb.download()
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    s0, r0 = pg.pagerank_static(ctx, ref)
    s1, r1 = pg.pagerank_static(ctx, mb)
    assert r0["iterations"] == r1["iterations"] and np.array_equal(s0, s1)
    ref.close()
    mb.close()


def test_batches_stop_at_an_untidy_batch(pg, ctx):
    xoff, xedg = _graph(pg, "rmat")
    batches = _batches(pg, xoff, xedg, 4, seed=30)
    # batch 2 deletes an edge that is not there
    n = len(xoff) - 1
    xo, xe = xoff, xedg
    for b in batches[:2]:
        xo, xe = pg.graphs.apply_batch(xo, xe, *b)
    u = 0
    row = set(xe[xo[u]:xo[u + 1]].tolist())
    v = next(w for w in range(n) if w not in row)
    du, dv, iu, iv = batches[2]
    keep = (du > u) | ((du == u) & (dv > v))
    bad = (np.concatenate([du[~keep], [u], du[keep]]).astype(np.uint32),
           np.concatenate([dv[~keep], [v], dv[keep]]).astype(np.uint32), iu, iv)
    xt = O.transpose(xoff, xedg)
    g = pg.Graph(ctx, *xt, xoff, xedg)
    q0, _ = pg.pagerank_static(ctx, g)
    with pytest.raises(pg.PrxError) as err:
        pg.solve_batches(ctx, g, pg.PRUNE_DYNAMIC_FRONTIER, [batches[0], batches[1], bad, batches[3]], q0)
    assert err.value.status == 1   # PRX_EINVAL
    got = g.download()
    assert np.array_equal(got[0], xo) and np.array_equal(got[1], xe)
    g.close()


def test_batches_argument_checks(pg, ctx):
    xoff, xedg = _graph(pg, "grid")
    xt = O.transpose(xoff, xedg)
    g = pg.Graph(ctx, *xt, xoff, xedg)
    q0, _ = pg.pagerank_static(ctx, g)
    b = _batches(pg, xoff, xedg, 1, seed=40)
    for mode in (pg.STATIC, pg.NAIVE_DYNAMIC, pg.DYNAMIC_TRAVERSAL):
        with pytest.raises(pg.PrxError):
            pg.solve_batches(ctx, g, mode, b, q0)
    with pytest.raises(pg.PrxError):
        pg.solve_batches(ctx, g, pg.DYNAMIC_FRONTIER, b, q0, opts=pg.options(precision=pg.FP32_REFINE))
    # ids out of range and lists out of order are caught on the device before
    # any row is read; the graph stays as it was
    n = len(xoff) - 1
    before = g.download()
    e = np.zeros(0, np.uint32)
    for bad in ((np.array([0], np.uint32), np.array([n], np.uint32), e, e),
                (e, e, np.array([3, 2], np.uint32), np.array([1, 1], np.uint32)),
                (e, e, np.array([2, 2], np.uint32), np.array([1, 1], np.uint32))):
        with pytest.raises(pg.PrxError) as err:
            pg.solve_batches(ctx, g, pg.DYNAMIC_FRONTIER, [bad], q0)
        assert err.value.status == 1
    assert all(np.array_equal(x, y) for x, y in zip(before, g.download()))
    # no batches: the ranks come back unchanged
    last, res, _ = pg.solve_batches(ctx, g, pg.DYNAMIC_FRONTIER, [], q0)
    assert res == [] and np.array_equal(last, q0)
    g.close()
    seg = pg.Graph.from_csr64(ctx, np.asarray(xt[0], np.uint64), xt[1], xt[2], np.asarray(xoff, np.uint64), xedg,
                              seg_shift=6)
    with pytest.raises(pg.PrxError) as err:
        pg.solve_batches(ctx, seg, pg.DYNAMIC_FRONTIER, b, q0)
    assert err.value.status == 5   # PRX_ERANGE
    seg.close()
