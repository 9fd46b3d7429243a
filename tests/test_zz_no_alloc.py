"""prx_static_solve_noalloc: the Static solve for callers that may not allocate
device memory (a process whose HBM is handed out only by its own allocator or
a fixed budget).  It must give the same ranks and iteration count as the
regular entry point, prx_solve(PRX_STATIC) -- bit for bit, the tolerance of
the other FP64 parity tests -- on consecutive calls that share its static
scratch, and refuse sizes beyond its limit.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1048576   # PRX_NOALLOC_MAX_VERTICES


def _lib():
    import pagerank_gb300 as pg
    lib = pg.load()
    f = lib.prx_static_solve_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int,
                  C.c_void_p, C.POINTER(C.c_int), C.c_void_p]
    return pg, f


def _reference_solution(pg, xt, **kw):
    with pg.Context(0) as ctx:
        g = pg.Graph(ctx, *xt)
        ranks, res = pg.solve(ctx, g, pg.STATIC, opts=pg.options(**kw))
        g.close()
    return ranks, res["iterations"]


def _noalloc(f, xt, damping=0.85, tol=1e-10, max_iter=500, stream=None, m=None):
    """One call; with `stream` (a torch.cuda.Stream) the inputs are made and
    the call is issued on that stream."""
    import torch
    with torch.cuda.stream(stream) if stream is not None else torch.cuda.device(0):
        xtoff, xtedg, xtdat = (torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
                               for a in xt)
        n = len(xt[0]) - 1
        m = len(xt[1]) if m is None else m
        ranks = torch.full((max(n, 1),), float("nan"), dtype=torch.float64, device="cuda")
    it = C.c_int(-1)
    if stream is None:
        torch.cuda.synchronize()
    st = f(n, m, xtoff.data_ptr(), xtedg.data_ptr(), xtdat.data_ptr(), damping, tol, max_iter, ranks.data_ptr(),
           C.byref(it), None if stream is None else stream.cuda_stream)
    torch.cuda.synchronize()
    return st, ranks[:n].cpu().numpy(), it.value


def test_noalloc_matches_regular_entry_point_on_consecutive_calls():
    pg, f = _lib()
    graphs = [pg.graphs.rmat(16, 16, seed=7),                       # 65,536 vertices, hubs above 64
              pg.graphs.weblike(300000, dmax=5000, window=512, seed=3),
              pg.graphs.rmat(16, 16, seed=7)]                      # the first graph again
    for off, edg in graphs:
        xt = pg.graphs.transpose(off, edg)
        want, want_it = _reference_solution(pg, xt)
        st, got, it = _noalloc(f, xt)
        assert st == 0, pg.load().prx_last_error()
        assert it == want_it
        np.testing.assert_array_equal(got, want)


def test_noalloc_options_and_limits():
    pg, f = _lib()
    off, edg = pg.graphs.rmat(10, 8, seed=5)
    xt = pg.graphs.transpose(off, edg)
    for kw, args in (({"max_iterations": 3}, {"max_iter": 3}), ({"damping": 0.5}, {"damping": 0.5}),
                     ({"max_iterations": 0}, {"max_iter": 0})):
        want, want_it = _reference_solution(pg, xt, **kw)
        st, got, it = _noalloc(f, xt, **args)
        assert st == 0 and it == want_it
        np.testing.assert_array_equal(got, want)
    # beyond the static scratch: refused before any device work
    it = C.c_int(-1)
    assert f(LIMIT + 1, 0, None, None, None, 0.85, 1e-10, 500, None, C.byref(it), None) == 5
    assert "exceeds" in pg.load().prx_last_error().decode()


def test_noalloc_on_a_non_default_stream():
    # inputs made on a torch stream and two calls issued on it back to back:
    # the stream argument is honoured and the second call re-initialises the
    # shared scratch the first one left behind
    import torch
    pg, f = _lib()
    off, edg = pg.graphs.rmat(15, 16, seed=9)
    xt = pg.graphs.transpose(off, edg)
    want, want_it = _reference_solution(pg, xt)
    s = torch.cuda.Stream()
    for _ in range(2):
        st, got, it = _noalloc(f, xt, stream=s)
        assert st == 0, pg.load().prx_last_error()
        assert it == want_it
        np.testing.assert_array_equal(got, want)


def test_noalloc_rejects_offsets_that_do_not_end_at_m():
    # xtoff[n] != m is caught on the device before any sweep; the next call
    # with the right m still gives the regular entry point's answer
    pg, f = _lib()
    off, edg = pg.graphs.rmat(10, 8, seed=5)
    xt = pg.graphs.transpose(off, edg)
    st, _, it = _noalloc(f, xt, m=len(xt[1]) - 1)
    assert st == 1 and it == 0
    assert "xtoff" in pg.load().prx_last_error().decode()
    want, want_it = _reference_solution(pg, xt)
    st, got, it = _noalloc(f, xt)
    assert st == 0 and it == want_it
    np.testing.assert_array_equal(got, want)
