"""GPU parity: the CUDA path (through the C ABI) against the oracle.

The FP64 path adds every in-edge contribution in the reference's order, so
ranks must be bit-identical to the oracle's GPU-semantics restatement and the
iteration counts equal; integer work (marking, batch apply) must be
bit-exact against the golden fixtures made by the reference's own code."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

MODES = ("static", "naive_dynamic", "dynamic_traversal", "dynamic_frontier", "prune_dynamic_frontier")


def _graph(pg, ctx, off, edg, xt=None):
    xtoff, xtedg, xtdat = xt if xt is not None else O.transpose(off, edg)
    return pg.Graph(ctx, xtoff, xtedg, xtdat, off, edg, validate=True), (xtoff, xtedg, xtdat)


def _oracle(mode, off, edg, xt, batch, q, opts=None):
    du, dv, iu, iv = batch
    return O.solve(mode, off, edg, *xt, du, dv, iu, iv, q=q, opts=opts)


def _gpu(pg, ctx, g, mode, batch, q, opts=None):
    du, dv, iu, iv = batch
    return pg.solve(ctx, g, pg.MODES[mode], (du, dv), (iu, iv), q, opts)


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    return pagerank_gb300


@pytest.mark.parametrize("case", golden_cases())
def test_golden_all_modes_bit_exact(pg, ctx, case):
    z = load_golden(case)
    batch = (z["del_u"], z["del_v"], z["ins_u"], z["ins_v"])
    xt = (z["yt_off"], z["yt_edg"], z["yt_dat"])
    g, _ = _graph(pg, ctx, z["y_off"], z["y_edg"], xt)
    q = z["static_x_ranks"]
    for mode in MODES:
        want, it_w = _oracle(mode, z["y_off"], z["y_edg"], xt, batch, q)
        got, res = _gpu(pg, ctx, g, mode, batch, q)
        assert res["iterations"] == it_w, mode
        np.testing.assert_array_equal(got, want, err_msg=mode)
    if int(z["n"]) > 1:
        assert np.abs(pg.pagerank_static(ctx, g)[0] - z["static_y_ranks"]).max() <= 1e-15
    g.close()


@pytest.mark.parametrize("case", golden_cases())
def test_golden_marking_bit_exact(pg, ctx, case):
    z = load_golden(case)
    g, _ = _graph(pg, ctx, z["y_off"], z["y_edg"], (z["yt_off"], z["yt_edg"], z["yt_dat"]))
    n = int(z["n"])
    dels, ins = (z["del_u"], z["del_v"]), (z["ins_u"], z["ins_v"])
    np.testing.assert_array_equal(pg.mark_affected(ctx, g, pg.DYNAMIC_FRONTIER, dels, ins), z["df_flags"][:n])
    np.testing.assert_array_equal(pg.mark_affected(ctx, g, pg.PRUNE_DYNAMIC_FRONTIER, dels, ins), z["df_flags"][:n])
    np.testing.assert_array_equal(pg.mark_affected(ctx, g, pg.DYNAMIC_TRAVERSAL, dels, ins), z["dt_flags"][:n])
    g.close()


@pytest.mark.parametrize("case", golden_cases())
def test_golden_device_batch_apply_bit_exact(pg, ctx, case):
    z = load_golden(case)
    g, _ = _graph(pg, ctx, z["x_off"], z["x_edg"], (z["xt_off"], z["xt_edg"], z["xt_dat"]))
    g.apply_batch(z["del_u"], z["del_v"], z["ins_u"], z["ins_v"])
    xoff, xedg, xtoff, xtedg, xtdat = g.download()
    for got, k in ((xoff, "y_off"), (xedg, "y_edg"), (xtoff, "yt_off"), (xtedg, "yt_edg"), (xtdat, "yt_dat")):
        np.testing.assert_array_equal(got, z[k], err_msg=k)
    # solving on the device-updated graph equals solving on the uploaded one
    q = z["static_x_ranks"]
    batch = (z["del_u"], z["del_v"], z["ins_u"], z["ins_v"])
    want, it = _oracle("prune_dynamic_frontier", z["y_off"], z["y_edg"], (z["yt_off"], z["yt_edg"], z["yt_dat"]),
                       batch, q)
    got, res = _gpu(pg, ctx, g, "prune_dynamic_frontier", batch, q)
    assert res["iterations"] == it
    np.testing.assert_array_equal(got, want)
    g.close()


def _synthetic(pg, kind):
    if kind == "rmat16":   # R-MAT scale 16 (65,536 vertices, 16 edges/vertex)
        return pg.graphs.rmat(16, 16, seed=42)
    if kind == "web200k":  # web-like, scaled down
        return pg.graphs.weblike(200000, dmax=20000, window=4096, seed=42)
    if kind == "grid256":  # road-like grid
        return pg.graphs.grid(256, 0.05, seed=42)
    if kind == "hubs":     # R-MAT with heavy hubs to exercise the HIGH class
        return pg.graphs.rmat(14, 48, a=0.7, b=0.1, c=0.1, seed=3)
    raise KeyError(kind)


@pytest.mark.parametrize("kind", ["rmat16", "web200k", "grid256", "hubs"])
def test_synthetic_all_modes_bit_exact(pg, ctx, kind):
    xoff, xedg = _synthetic(pg, kind)
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, max(1, int(2e-5 * m)), max(1, int(8e-5 * m)), seed=11)
    xt = O.transpose(xoff, xedg)
    q, _ = O.solve("static", None, None, *xt)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    g, _ = _graph(pg, ctx, xoff, xedg, xt)
    g.apply_batch(*batch)       # the device applies the batch to both CSRs
    for mode in MODES:
        want, it_w = _oracle(mode, yoff, yedg, yt, batch, q)
        got, res = _gpu(pg, ctx, g, mode, batch, q)
        assert res["iterations"] == it_w, (kind, mode)
        np.testing.assert_array_equal(got, want, err_msg=f"{kind} {mode}")
    g.close()


@pytest.mark.parametrize("kind", ["rmat16", "web200k"])
def test_frontier_expansion_push_and_pull_agree(pg, ctx, kind):
    # DF / DF-P mark the out-neighbours of every vertex whose change exceeded
    # D; pushing from those vertices and pulling into the unmarked ones must
    # give the oracle's ranks bit for bit, on a batch large enough that many
    # vertices change in the first iterations.
    xoff, xedg = _synthetic(pg, kind)
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, int(5e-4 * m), int(2e-3 * m), seed=5)
    xt = O.transpose(xoff, xedg)
    q, _ = O.solve("static", None, None, *xt)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    g, _ = _graph(pg, ctx, yoff, yedg, yt)
    # DT: the closure by push levels, by pull rounds, or switching between them
    for mode in ("dynamic_frontier", "prune_dynamic_frontier", "dynamic_traversal"):
        want, it_w = _oracle(mode, yoff, yedg, yt, batch, q)
        for expansion in (0, 1, 2):
            got, res = _gpu(pg, ctx, g, mode, batch, q, pg.options(expansion=expansion))
            assert res["iterations"] == it_w, (kind, mode, expansion)
            np.testing.assert_array_equal(got, want, err_msg=f"{kind} {mode} expansion={expansion}")
    g.close()


@pytest.mark.parametrize("kind,width", [("rmat16", 1000), ("rmat16", 20000), ("web200k", 7777),
                                        ("hubs", 3000), ("grid256", 5000)])
def test_chunked_gathers_bit_exact(pg, ctx, kind, width):
    # The in-degree <= 64 class gathers its contributions one source chunk at a
    # time, carrying the row sum between chunks; rows are sorted by source, so
    # every chunk width must reproduce the reference's sequential order.
    xoff, xedg = _synthetic(pg, kind)
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, max(1, int(2e-4 * m)), max(1, int(8e-4 * m)), seed=13)
    xt = O.transpose(xoff, xedg)
    q, _ = O.solve("static", None, None, *xt)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    g, _ = _graph(pg, ctx, yoff, yedg, yt)
    opts = pg.options(chunk_vertices=width)
    for mode in MODES:
        want, it_w = _oracle(mode, yoff, yedg, yt, batch, q)
        got, res = _gpu(pg, ctx, g, mode, batch, q, opts)
        assert res["iterations"] == it_w, (kind, width, mode)
        np.testing.assert_array_equal(got, want, err_msg=f"{kind} width={width} {mode}")
    want, _ = O.solve("static", None, None, *yt)
    got, _ = pg.solve(ctx, g, pg.STATIC, opts=pg.options(chunk_vertices=width, precision=pg.FP32_REFINE))
    assert np.abs(got - want).max() <= 1e-9
    g.close()


@pytest.mark.parametrize("kind", ["rmat16", "web200k", "hubs", "grid256"])
def test_hot_sources_bit_exact(pg, ctx, kind):
    # Static / ND and the refinement's FP64 sweeps gather the contributions of
    # the highest out-degree vertices from a dense copy (hot_sources: 0 the
    # default cap, -1 none, k at most k vertices); the values are the same, so
    # every cap, chunk width and loop gives the oracle's ranks bit for bit,
    # also after a batch changes the degrees (the hot set is rebuilt)
    xoff, xedg = _synthetic(pg, kind)
    xt = O.transpose(xoff, xedg)
    g, _ = _graph(pg, ctx, xoff, xedg, xt)
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, max(1, int(2e-4 * m)), max(1, int(8e-4 * m)), seed=29)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    for graph_t in (xt, yt):
        want, it_w = O.solve("static", None, None, *graph_t)
        q = want * (1 + 1e-3 * np.cos(np.arange(len(want))))
        nd_want, nd_it = O.solve("naive_dynamic", None, None, *graph_t, q=q)
        for cap in (0, -1, 1, 100, 5000):
            for width in (0, 997, 10 ** 9):
                for loop in (pg.LOOP_AUTO, pg.LOOP_HOST):
                    o = pg.options(hot_sources=cap, chunk_vertices=width, loop=loop)
                    got, res = pg.solve(ctx, g, pg.STATIC, opts=o)
                    assert res["iterations"] == it_w, (kind, cap, width, loop)
                    np.testing.assert_array_equal(got, want, err_msg=f"{kind} cap={cap} width={width}")
                    got, res = pg.solve(ctx, g, pg.NAIVE_DYNAMIC, q=q, opts=o)
                    assert res["iterations"] == nd_it
                    np.testing.assert_array_equal(got, nd_want, err_msg=f"{kind} ND cap={cap} width={width}")
                got, _ = pg.solve(ctx, g, pg.STATIC, opts=pg.options(hot_sources=cap, chunk_vertices=width,
                                                                     precision=pg.FP32_REFINE))
                assert np.abs(got - want).max() <= 1e-9
        if graph_t is xt:
            g.apply_batch(*batch)
    with pytest.raises(Exception):
        pg.solve(ctx, g, pg.STATIC, opts=pg.options(hot_sources=-2))
    g.close()


@pytest.mark.parametrize("kind", ["web200k", "hubs"])
def test_host_and_graph_loops_agree(pg, ctx, kind):
    # the iteration loop as one CUDA graph (conditional while node) and the
    # host-driven loop give the oracle's ranks and iteration counts, also
    # under small iteration caps
    xoff, xedg = _synthetic(pg, kind)
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, max(1, int(2e-4 * m)), max(1, int(8e-4 * m)), seed=23)
    xt = O.transpose(xoff, xedg)
    q, _ = O.solve("static", None, None, *xt)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    g, _ = _graph(pg, ctx, yoff, yedg, yt)
    for cap in (500, 0, 1, 3):
        for mode in MODES:
            want, it_w = _oracle(mode, yoff, yedg, yt, batch, q, O.options(max_iterations=cap))
            for loop in (pg.LOOP_HOST, pg.LOOP_GRAPH):
                got, res = _gpu(pg, ctx, g, mode, batch, q, pg.options(loop=loop, max_iterations=cap))
                assert res["iterations"] == it_w, (kind, mode, cap, loop)
                np.testing.assert_array_equal(got, want, err_msg=f"{kind} {mode} cap={cap} loop={loop}")
    g.close()


def test_graph_outlives_context(pg):
    # destroying a context first must leave its graphs destroyable
    c = pg.Context(0)
    xoff, xedg = pg.graphs.rmat(8, 8, seed=2)
    g = pg.Graph(c, *O.transpose(xoff, xedg))
    c.close()
    g.close()


def test_options_edge_cases(pg, ctx):
    xoff, xedg = pg.graphs.rmat(10, 16, seed=1)
    xt = O.transpose(xoff, xedg)
    g, _ = _graph(pg, ctx, xoff, xedg, xt)
    for kw in ({"max_iterations": 0}, {"max_iterations": 1}, {"max_iterations": 7}, {"tolerance": 1.0},
               {"tolerance": 1e-14}, {"damping": 0.5}, {"repeat": 3}):
        opts = pg.options(**kw)
        oo = O.options(**{k: v for k, v in kw.items() if k != "repeat"})
        want, it = O.solve("static", None, None, *xt, opts=oo)
        got, res = pg.solve(ctx, g, pg.STATIC, opts=opts)
        assert res["iterations"] == it, kw
        np.testing.assert_array_equal(got, want, err_msg=str(kw))
    g.close()


def test_empty_batch_and_empty_graph(pg, ctx):
    xoff, xedg = pg.graphs.rmat(9, 8, seed=1)
    xt = O.transpose(xoff, xedg)
    g, _ = _graph(pg, ctx, xoff, xedg, xt)
    q = np.full(len(xoff) - 1, 1.0 / (len(xoff) - 1))
    e = np.zeros(0, np.uint32)
    for mode in MODES[2:]:
        got, res = pg.solve(ctx, g, pg.MODES[mode], (e, e), (e, e), q)
        assert res["iterations"] == 1 and res["affected_initial"] == 0
        np.testing.assert_array_equal(got, q)
    g.close()
    z = np.zeros(1, np.uint32)
    g0 = pg.Graph(ctx, z, np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    r, res = pg.solve(ctx, g0, pg.STATIC)
    assert len(r) == 0 and res["iterations"] == 0
    g0.close()


def test_errors_are_status_codes(pg, ctx):
    xoff, xedg = pg.graphs.rmat(8, 8, seed=1)
    xtoff, xtedg, xtdat = O.transpose(xoff, xedg)
    g = pg.Graph(ctx, xtoff, xtedg, xtdat)       # no out-CSR
    with pytest.raises(pg.PrxError) as e:
        pg.solve(ctx, g, pg.DYNAMIC_FRONTIER, (np.zeros(0), np.zeros(0)), ([1], [2]), None)
    assert e.value.status == 6
    g.close()
    g = pg.Graph(ctx, xtoff, xtedg, xtdat, xoff, xedg)
    with pytest.raises(pg.PrxError) as e:             # vertex id out of range
        pg.solve(ctx, g, pg.DYNAMIC_FRONTIER, ([0], [10 ** 6]), ([0], [1]), None)
    assert e.value.status == 1
    with pytest.raises(pg.PrxError) as e:             # insertion of an existing edge: not tidy
        g.apply_batch([], [], [0], [0])
    assert e.value.status == 1
    bad = xtedg.copy()
    bad[0] = 10 ** 6
    with pytest.raises(pg.PrxError):
        pg.Graph(ctx, xtoff, bad, xtdat, validate=True)
    g.close()


def test_reciprocal_division_matches_ieee(pg, ctx):
    # The solvers form contributions r / outdeg as q = r*y, r' = fma(-q, d, r),
    # fma(r', y, q) with y = 1/d precomputed; it must equal the IEEE quotient
    # bit for bit: every out-degree 1 .. 2^17 with 256 dividends each, and a
    # sparser sweep of large out-degrees.
    assert pg.selftest_division(ctx, 1 << 17, 256) == 0
    assert pg.selftest_division(ctx, 1 << 24, 4) == 0


def test_autotune_keeps_results_and_caches(pg, ctx, tmp_path):
    # the tuner only picks execution parameters: ranks and iteration counts
    # stay the oracle's; a graph of the same signature reuses the picks, also
    # through the cache file
    xoff, xedg = _synthetic(pg, "hubs")
    m = len(xedg)
    batch = pg.graphs.random_batch(xoff, xedg, max(1, int(2e-4 * m)), max(1, int(8e-4 * m)), seed=37)
    xt = O.transpose(xoff, xedg)
    q, _ = O.solve("static", None, None, *xt)
    yoff, yedg = pg.graphs.apply_batch(xoff, xedg, *batch)
    yt = O.transpose(yoff, yedg)
    g, _ = _graph(pg, ctx, yoff, yedg, yt)
    path = tmp_path / "tune.txt"
    t = pg.autotune(ctx, g, path)
    assert t["trials"] > 0 and t["cached"] == 0 and t["mid_max"] in (1024, 4096, 16384)
    for mode in MODES:
        want, it_w = _oracle(mode, yoff, yedg, yt, batch, q)
        got, res = _gpu(pg, ctx, g, mode, batch, q)
        assert res["iterations"] == it_w, mode
        np.testing.assert_array_equal(got, want, err_msg=mode)
    g2, _ = _graph(pg, ctx, yoff, yedg, yt)
    # built after the tuning: the picks (here the MID / HIGH split) are taken at creation
    assert g2.class_stats() == g.class_stats()
    t2 = pg.autotune(ctx, g2)
    assert t2["cached"] == 1 and t2["trials"] == 0 and t2["mid_max"] == t["mid_max"]
    assert t["l2_fetch_bytes"] in (32, 64, 128) and t2["l2_fetch_bytes"] == t["l2_fetch_bytes"]
    assert t["int_adds"] in (-1, 1, 2, 3, 4) and t2["int_adds"] == t["int_adds"]
    lines = path.read_text().split()
    assert len(lines) >= 8 and int(lines[1]) == t["mid_max"] and int(lines[6]) == t["l2_fetch_bytes"]
    assert int(lines[7]) == t["int_adds"]
    g2.close()
    g.close()


def test_require_convergence_reports_the_cap(pg, ctx):
    # opt-in PRX_ENOCONV: a solve cut by the iteration cap says so; one that
    # converges returns as without the flag
    xoff, xedg = _synthetic(pg, "hubs")
    xt = O.transpose(xoff, xedg)
    g, _ = _graph(pg, ctx, xoff, xedg, xt)
    want, it = O.solve("static", None, None, *xt)
    assert it > 3
    got, res = pg.pagerank_static(ctx, g, opts=pg.options(require_convergence=1))
    assert res["iterations"] == it and np.array_equal(got, want) and res["last_delta"] < 1e-10
    with pytest.raises(pg.PrxError) as e:
        pg.pagerank_static(ctx, g, opts=pg.options(require_convergence=1, max_iterations=3))
    assert e.value.status == 7
    _, res3 = pg.pagerank_static(ctx, g, opts=pg.options(max_iterations=3))
    assert res3["iterations"] == 3 and res3["last_delta"] >= 1e-10
    g.close()


def test_l2_fetch_granularity_is_restored_and_changes_nothing(pg, ctx):
    # the solve sets the hint for its own duration only; every granularity
    # gives the oracle's ranks bit for bit
    xoff, xedg = _synthetic(pg, "hubs")
    xt = O.transpose(xoff, xedg)
    g, _ = _graph(pg, ctx, xoff, xedg, xt)
    want, it_w = O.solve("static", None, None, *xt)
    prev = pg.l2_fetch_granularity()
    assert pg.l2_fetch_granularity(128) == prev and pg.l2_fetch_granularity() == 128
    pg.l2_fetch_granularity(prev)
    for f in (-1, 0, 32, 64, 128):
        got, res = pg.pagerank_static(ctx, g, opts=pg.options(l2_fetch_bytes=f))
        assert res["iterations"] == it_w
        np.testing.assert_array_equal(got, want)
        assert pg.l2_fetch_granularity() == prev, f
    for bad in (-2, 129):
        with pytest.raises(pg.PrxError) as e:
            pg.pagerank_static(ctx, g, opts=pg.options(l2_fetch_bytes=bad))
        assert e.value.status == 1
    with pytest.raises(pg.PrxError):
        pg.l2_fetch_granularity(129)
    assert pg.l2_fetch_granularity() == prev
    g.close()


@pytest.mark.parametrize("case", golden_cases())
def test_device_tidy_matches_reference_golden(pg, ctx, case):
    # the raw batch tidied on the device against x equals the reference's own
    # tidyBatchUpdateU output stored in the fixture
    z = load_golden(case)
    g = pg.Graph(ctx, z["xt_off"], z["xt_edg"], z["xt_dat"], z["x_off"], z["x_edg"])
    du, dv, iu, iv = g.tidy_batch(z["raw_del_u"], z["raw_del_v"], z["raw_ins_u"], z["raw_ins_v"])
    np.testing.assert_array_equal(du, z["del_u"])
    np.testing.assert_array_equal(dv, z["del_v"])
    np.testing.assert_array_equal(iu, z["ins_u"])
    np.testing.assert_array_equal(iv, z["ins_v"])
    g.close()


@pytest.mark.parametrize("kind", ["rmat16", "hubs", "web200k"])
def test_device_tidy_matches_host_tidy(pg, ctx, kind):
    xoff, xedg = _synthetic(pg, kind)
    n, m = len(xoff) - 1, len(xedg)
    rng = np.random.default_rng(41)
    src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(xoff.astype(np.int64)))
    pick = rng.integers(0, m, 30000)
    # deletions: existing edges with repeats, plus random pairs (mostly absent)
    du = np.concatenate([src[pick], rng.integers(0, n, 5000).astype(np.uint32)])
    dv = np.concatenate([xedg[pick], rng.integers(0, n, 5000).astype(np.uint32)])
    # insertions: random pairs with repeats, plus some existing edges
    iu0 = rng.integers(0, n, 40000).astype(np.uint32)
    iv0 = rng.integers(0, n, 40000).astype(np.uint32)
    iu = np.concatenate([iu0, iu0[:3000], src[pick[:2000]]])
    iv = np.concatenate([iv0, iv0[:3000], xedg[pick[:2000]]])
    perm = rng.permutation(len(du))
    du, dv = du[perm], dv[perm]
    g = pg.Graph(ctx, *O.transpose(xoff, xedg), xoff, xedg)
    got = g.tidy_batch(du, dv, iu, iv)
    want = pg.graphs.tidy_batch(xoff, xedg, du, dv, iu, iv)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
    g.apply_batch(*got)  # the result is a valid batch for the device apply
    e = np.zeros(0, np.uint32)
    assert all(len(a) == 0 for a in g.tidy_batch(e, e, e, e))
    g.close()


@pytest.mark.parametrize("kind", ["rmat", "grid"])
def test_device_batch_generation_matches_host(pg, ctx, kind):
    """prx_graph_gen_batch draws the same raw batch as the host generator
    (same counter-based hashes) and tidies it on the device."""
    if kind == "rmat":
        xoff, xedg = pg.graphs.rmat(14, 8, seed=3)
    else:
        xoff, xedg = pg.graphs.grid(128, seed=3)
    g = pg.Graph.from_out_csr(ctx, xoff, xedg)
    for nd, ni, seed in [(0, 0, 1), (5, 0, 2), (0, 7, 3), (300, 1200, 4), (20000, 80000, 5)]:
        want = pg.graphs.random_batch(xoff, xedg, nd, ni, seed=seed)
        got = g.gen_batch(nd, ni, seed=seed)
        for a, b in zip(got, want):
            assert np.array_equal(a, b), (nd, ni, seed)
    g.close()


def test_graph_pool_reuse_and_release(pg, ctx):
    """Graphs built one after another reuse the pool's memory; results do not
    change, and releasing the cached memory leaves later graphs working."""
    xoff, xedg = pg.graphs.rmat(14, 8, seed=5)
    xt = O.transpose(xoff, xedg)
    want, it = O.solve("static", None, None, *xt)
    for k in range(3):
        s0 = pg.graph_pool_stats()
        g = pg.Graph(ctx, *xt, xoff, xedg)
        s1 = pg.graph_pool_stats()
        assert s1["used"] >= s0["used"] + 8 * len(xedg) and s1["reserved"] >= s1["used"]
        assert s1["reserved_peak"] >= s1["reserved"] and s1["used_peak"] >= s1["used"]
        r, res = pg.pagerank_static(ctx, g, pg.options(chunk_vertices=4096))
        assert res["iterations"] == it and np.array_equal(r, want)
        g.close()
        if k:  # (the first solve may add the context's own pool buffers)
            assert pg.graph_pool_stats()["used"] == s0["used"]
        if k == 1:
            pg.release_cached_memory(0)
            assert pg.graph_pool_stats()["reserved"] <= s1["reserved"]
