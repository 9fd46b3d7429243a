"""Python face of the C ABI: contexts, device graphs, solves.

Mirrors the reference's solver surface (inc/pagerankCuda.hxx:864-988):

    pagerank_static(ctx, g, options)                          pagerankStaticCuda
    pagerank_naive_dynamic(ctx, g, q, options)                pagerankNaiveDynamicCuda
    pagerank_dynamic_traversal(ctx, g, dels, ins, q, options) pagerankDynamicTraversalCuda
    pagerank_dynamic_frontier(ctx, g, dels, ins, q, options)  pagerankDynamicFrontierCuda
    pagerank_prune_dynamic_frontier(...)                      pagerankPruneDynamicFrontierCuda

each returning (ranks, PagerankResult-like dict).  The graph passed is the
updated graph y (with its transpose), as the reference's callers pass it.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import Options, PprResult, Result, TuneResult, check, load


def options(**kw):
    o = Options()
    load().prx_options_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown option {k}")
        setattr(o, k, v)
    return o


def _u32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.uint32)


def _p(a):
    return None if a is None or len(a) == 0 else a.ctypes.data


class Context:
    """prx_context: one CUDA device + stream + workspace."""

    def __init__(self, device=0):
        self._h = C.c_void_p()
        self.device = device
        check(load().prx_context_create(device, C.byref(self._h)), "prx_context_create")

    @property
    def handle(self):
        return self._h

    @property
    def stream(self):
        return load().prx_context_stream(self._h)

    def close(self):
        if self._h:
            load().prx_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Graph:
    """prx_graph: device CSR of a graph and its transpose (+ out-degrees)."""

    def __init__(self, ctx, xtoff, xtedg, xtdat, xoff=None, xedg=None, validate=False):
        xtoff, xtedg, xtdat, xoff, xedg = (_u32(a) for a in (xtoff, xtedg, xtdat, xoff, xedg))
        self.ctx = ctx
        self._h = C.c_void_p()
        n, m = len(xtoff) - 1, len(xtedg)
        check(load().prx_graph_create(ctx.handle, n, m, _p(xoff), _p(xedg) if xoff is not None else None,
                                      xtoff.ctypes.data, _p(xtedg), _p(xtdat), int(validate), C.byref(self._h)),
              "prx_graph_create")

    @classmethod
    def from_out_csr(cls, ctx, off, edg, dynamic=True, validate=False):
        from .graphs import transpose
        xtoff, xtedg, xtdat = transpose(off, edg)
        return cls(ctx, xtoff, xtedg, xtdat, off if dynamic else None, edg if dynamic else None, validate)

    @classmethod
    def from_edges(cls, ctx, n, u, v, self_loops=True):
        """prx_graph_create_from_edges: sort, merge and transpose an edge list
        (0-based ids < n) on the device, with a self-loop on every vertex when
        self_loops is set (main.cu:167-170 of the reference, on the host there)."""
        u, v = _u32(u), _u32(v)
        if len(u) != len(v):
            raise ValueError("u and v differ in length")
        g = cls.__new__(cls)
        g.ctx = ctx
        g._h = C.c_void_p()
        check(load().prx_graph_create_from_edges(ctx.handle, int(n), _p(u), _p(v), len(u), int(bool(self_loops)),
                                                 C.byref(g._h)), "prx_graph_create_from_edges")
        return g

    @classmethod
    def from_csr64(cls, ctx, xtoff, xtedg, xtdat, xoff=None, xedg=None, seg_shift=0, validate=False):
        """prx_graph_create64: 64-bit offsets (graphs of 2^32 edges or more);
        seg_shift 0 picks the row segments, 1..32 forces them."""
        xtoff = np.ascontiguousarray(xtoff, dtype=np.uint64)
        xoff = None if xoff is None else np.ascontiguousarray(xoff, dtype=np.uint64)
        xtedg, xtdat, xedg = (_u32(a) for a in (xtedg, xtdat, xedg))
        g = cls._wrap(ctx)
        n, m = len(xtoff) - 1, len(xtedg)
        check(load().prx_graph_create64(ctx.handle, n, m, _p(xoff), _p(xedg) if xoff is not None else None,
                                        xtoff.ctypes.data, _p(xtedg), _p(xtdat), int(validate), int(seg_shift),
                                        C.byref(g._h)), "prx_graph_create64")
        return g

    def download64(self, out_csr=True):
        """prx_graph_download64 -> (xoff, xedg, xtoff, xtedg, xtdat) with 64-bit offsets."""
        n, m = self.size()
        xoff = np.zeros(n + 1, np.uint64) if out_csr else None
        xedg = np.zeros(max(m, 1), np.uint32) if out_csr else None
        xtoff, xtedg = np.zeros(n + 1, np.uint64), np.zeros(max(m, 1), np.uint32)
        xtdat = np.zeros(max(n, 1), np.uint32)
        check(load().prx_graph_download64(self._h, None if xoff is None else xoff.ctypes.data,
                                          None if xedg is None else xedg.ctypes.data, xtoff.ctypes.data,
                                          xtedg.ctypes.data, xtdat.ctypes.data), "prx_graph_download64")
        return xoff, None if xedg is None else xedg[:m], xtoff, xtedg[:m], xtdat[:n]

    @classmethod
    def _wrap(cls, ctx):
        g = cls.__new__(cls)
        g.ctx = ctx
        g._h = C.c_void_p()
        return g

    @classmethod
    def from_text(cls, ctx, text, rows, size=None, symmetric=False, self_loops=True):
        """prx_graph_create_from_text: SNAP temporal text (bytes, 1-based ids)
        parsed and built on the device -> (graph, lines consumed, bytes consumed)."""
        if not isinstance(text, bytes):
            text = bytes(text)
        g = cls._wrap(ctx)
        lines, used = C.c_uint64(), C.c_uint64()
        size = (1 << 64) - 1 if size is None else int(size)
        check(load().prx_graph_create_from_text(ctx.handle, text, len(text), int(rows), size,
                                                int(bool(symmetric)), int(bool(self_loops)), C.byref(g._h),
                                                C.byref(lines), C.byref(used)), "prx_graph_create_from_text")
        return g, lines.value, used.value

    @classmethod
    def from_reader(cls, ctx, reader, rows, size, symmetric=False, self_loops=True):
        """prx_edge_reader_next_graph: the next `size` lines of an EdgeReader,
        parsed and built on the device -> (graph, lines consumed)."""
        g = cls._wrap(ctx)
        lines = C.c_uint64()
        check(load().prx_edge_reader_next_graph(reader._h, ctx.handle, int(rows), int(size), int(bool(symmetric)),
                                                int(bool(self_loops)), C.byref(g._h), C.byref(lines)),
              "prx_edge_reader_next_graph")
        return g, lines.value

    @classmethod
    def from_mtx(cls, ctx, path, self_loops=True):
        """prx_graph_create_from_mtx: a MatrixMarket coordinate file parsed and
        built on the device -> (graph, n)."""
        g = cls._wrap(ctx)
        n = C.c_uint32()
        check(load().prx_graph_create_from_mtx(ctx.handle, str(path).encode(), int(bool(self_loops)),
                                               C.byref(g._h), C.byref(n)), "prx_graph_create_from_mtx")
        return g, n.value

    @classmethod
    def from_device_edges(cls, ctx, n, u, v, self_loops=True):
        """prx_graph_create_from_edges_device: u, v are int32/uint32 CUDA
        tensors (torch) of equal length, already resident on the device."""
        if u.numel() != v.numel() or u.element_size() != 4 or v.element_size() != 4:
            raise ValueError("u and v must be 4-byte integer tensors of equal length")
        if not (u.is_cuda and v.is_cuda and u.is_contiguous() and v.is_contiguous()):
            raise ValueError("u and v must be contiguous CUDA tensors")
        import torch
        torch.cuda.current_stream(u.device).synchronize()   # the library works on its own stream
        g = cls.__new__(cls)
        g.ctx = ctx
        g._h = C.c_void_p()
        check(load().prx_graph_create_from_edges_device(ctx.handle, int(n), u.data_ptr() or None,
                                                        v.data_ptr() or None, u.numel(), int(bool(self_loops)),
                                                        C.byref(g._h)), "prx_graph_create_from_edges_device")
        return g

    @property
    def handle(self):
        return self._h

    def size(self):
        n, m = C.c_uint32(), C.c_uint64()
        check(load().prx_graph_size(self._h, C.byref(n), C.byref(m)), "prx_graph_size")
        return n.value, m.value

    def class_stats(self):
        """(vertices[3], in-edges[3]) per in-degree class of the rank update."""
        nv, ne = (C.c_uint32 * 3)(), (C.c_uint64 * 3)()
        check(load().prx_graph_class_stats(self._h, nv, ne), "prx_graph_class_stats")
        return list(nv), list(ne)

    def apply_batch(self, del_u, del_v, ins_u, ins_v):
        du, dv, iu, iv = (_u32(a) for a in (del_u, del_v, ins_u, ins_v))
        check(load().prx_graph_apply_batch(self._h, _p(du), _p(dv), len(du), _p(iu), _p(iv), len(iu)),
              "prx_graph_apply_batch")

    def tidy_batch(self, del_u, del_v, ins_u, ins_v):
        """prx_graph_tidy_batch: the tidied (del_u, del_v, ins_u, ins_v) for this graph."""
        du, dv, iu, iv = (_u32(a) for a in (del_u, del_v, ins_u, ins_v))
        od, odv = np.zeros(max(len(du), 1), np.uint32), np.zeros(max(len(du), 1), np.uint32)
        oi, oiv = np.zeros(max(len(iu), 1), np.uint32), np.zeros(max(len(iu), 1), np.uint32)
        nd, ni = C.c_uint64(), C.c_uint64()
        check(load().prx_graph_tidy_batch(self.ctx.handle, self._h, _p(du), _p(dv), len(du), _p(iu), _p(iv), len(iu),
                                          od.ctypes.data, odv.ctypes.data, C.byref(nd), oi.ctypes.data,
                                          oiv.ctypes.data, C.byref(ni)), "prx_graph_tidy_batch")
        return od[:nd.value], odv[:nd.value], oi[:ni.value], oiv[:ni.value]

    def gen_batch(self, n_del, n_ins, seed=7):
        """prx_graph_gen_batch: a random batch drawn and tidied on the device ->
        (del_u, del_v, ins_u, ins_v); the same as graphs.random_batch on this
        graph's out-CSR."""
        od, odv = np.zeros(max(n_del, 1), np.uint32), np.zeros(max(n_del, 1), np.uint32)
        oi, oiv = np.zeros(max(n_ins, 1), np.uint32), np.zeros(max(n_ins, 1), np.uint32)
        nd, ni = C.c_uint64(), C.c_uint64()
        check(load().prx_graph_gen_batch(self.ctx.handle, self._h, int(n_del), int(n_ins), int(seed), od.ctypes.data,
                                         odv.ctypes.data, C.byref(nd), oi.ctypes.data, oiv.ctypes.data,
                                         C.byref(ni)), "prx_graph_gen_batch")
        return od[:nd.value], odv[:nd.value], oi[:ni.value], oiv[:ni.value]

    def download(self):
        n, m = self.size()
        xoff, xtoff = np.zeros(n + 1, np.uint32), np.zeros(n + 1, np.uint32)
        xedg, xtedg = np.zeros(max(m, 1), np.uint32), np.zeros(max(m, 1), np.uint32)
        xtdat = np.zeros(max(n, 1), np.uint32)
        check(load().prx_graph_download(self._h, xoff.ctypes.data, xedg.ctypes.data, xtoff.ctypes.data,
                                        xtedg.ctypes.data, xtdat.ctypes.data), "prx_graph_download")
        return xoff, xedg[:m], xtoff, xtedg[:m], xtdat[:n]

    def close(self):
        if self._h:
            load().prx_graph_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve(ctx, g, mode, deletions=None, insertions=None, q=None, opts=None):
    """prx_solve with host buffers -> (ranks float64[n], result dict)."""
    n, _ = g.size()
    du = dv = iu = iv = None
    if deletions is not None:
        du, dv = _u32(deletions[0]), _u32(deletions[1])
    if insertions is not None:
        iu, iv = _u32(insertions[0]), _u32(insertions[1])
    qq = None if q is None else np.ascontiguousarray(q, dtype=np.float64)
    if qq is not None and len(qq) != n:
        raise ValueError("q must have one entry per vertex")
    ranks = np.zeros(max(n, 1), np.float64)
    res = Result()
    check(load().prx_solve(ctx.handle, g.handle, int(mode), _p(du), _p(dv), 0 if du is None else len(du),
                           _p(iu), _p(iv), 0 if iu is None else len(iu), _p(qq), C.byref(opts or options()),
                           ranks.ctypes.data, C.byref(res)), "prx_solve")
    return ranks[:n], res.as_dict()


def solve_into(ctx, g, mode, ranks_host_ptr, q_host_ptr=None, opts=None):
    """prx_solve into a caller-owned host buffer (e.g. pinned memory) -> result dict."""
    res = Result()
    check(load().prx_solve(ctx.handle, g.handle, int(mode), None, None, 0, None, None, 0, q_host_ptr,
                           C.byref(opts or options()), ranks_host_ptr, C.byref(res)), "prx_solve")
    return res.as_dict()


def solve_device(ctx, g, mode, q_ptr, ranks_ptr, batch_ptrs=(None, None, 0, None, None, 0), opts=None):
    """prx_solve_device with device pointers (ints) -> result dict."""
    du, dv, nd, iu, iv, ni = batch_ptrs
    res = Result()
    check(load().prx_solve_device(ctx.handle, g.handle, int(mode), du, dv, nd, iu, iv, ni, q_ptr,
                                  C.byref(opts or options()), ranks_ptr, C.byref(res)), "prx_solve_device")
    return res.as_dict()


def solve_batches(ctx, g, mode, batches, q, opts=None, each=False):
    """prx_solve_batches_device: apply and solve K consecutive batches
    [(del_u, del_v, ins_u, ins_v), ...] as one CUDA graph launch, from ranks q
    -> (ranks after the last batch, [result dict per batch], ranks per batch
    float64[K, n] or None).  Host arrays in and out (copied through device
    tensors)."""
    import torch
    n, _ = g.size()
    K = len(batches)
    dev = torch.device("cuda", ctx.device)
    lists = [[_u32(b[i]) for b in batches] for i in range(4)]
    del_off = np.zeros(K + 1, np.uint64)
    ins_off = np.zeros(K + 1, np.uint64)
    del_off[1:] = np.cumsum([len(x) for x in lists[0]])
    ins_off[1:] = np.cumsum([len(x) for x in lists[2]])

    def up(parts):
        a = np.concatenate(parts) if parts else np.zeros(0, np.uint32)
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int32).copy()).to(dev)

    du, dv, iu, iv = (up(x) for x in lists)
    qd = torch.from_numpy(np.ascontiguousarray(q, dtype=np.float64).copy()).to(dev)
    out = torch.empty(max(n, 1), dtype=torch.float64, device=dev)
    each_d = torch.empty((K, max(n, 1)), dtype=torch.float64, device=dev) if each and K else None
    res = (Result * max(K, 1))()
    done = C.c_uint32()
    torch.cuda.current_stream(dev).synchronize()   # the library works on its own stream
    st = load().prx_solve_batches_device(ctx.handle, g.handle, int(mode), K, del_off.ctypes.data,
                                         du.data_ptr() or None, dv.data_ptr() or None, ins_off.ctypes.data,
                                         iu.data_ptr() or None, iv.data_ptr() or None, qd.data_ptr(),
                                         C.byref(opts or options()), out.data_ptr(),
                                         None if each_d is None else each_d.data_ptr(), res, C.byref(done))
    results = [res[k].as_dict() for k in range(done.value)]
    check(st, "prx_solve_batches_device")
    return (out.cpu().numpy()[:n], results, None if each_d is None else each_d.cpu().numpy()[:, :n])


def release_cached_memory(device=0):
    """prx_release_cached_memory: give the graph pool's free memory on a device back to the driver."""
    check(load().prx_release_cached_memory(int(device)), "prx_release_cached_memory")


def graph_pool_stats(device=0):
    """prx_graph_pool_stats -> dict of the graph pool's reserved / used bytes (now and peak)."""
    v = [C.c_uint64() for _ in range(4)]
    check(load().prx_graph_pool_stats(int(device), *(C.byref(x) for x in v)), "prx_graph_pool_stats")
    return dict(zip(("reserved", "reserved_peak", "used", "used_peak"), (x.value for x in v)))


def l2_fetch_granularity(bytes_=None, device=0):
    """prx_l2_fetch_granularity: the previous L2 fetch granularity hint of this
    process on `device`; sets it to bytes_ (0..128) when given."""
    prev = C.c_int32()
    check(load().prx_l2_fetch_granularity(int(device), -1 if bytes_ is None else int(bytes_), C.byref(prev)),
          "prx_l2_fetch_granularity")
    return prev.value


def mark_affected(ctx, g, mode, deletions, insertions):
    """Initial affected flags of a dynamic mode -> uint8[n]."""
    n, _ = g.size()
    du, dv = _u32(deletions[0]), _u32(deletions[1])
    iu = _u32(insertions[0])
    flags = np.zeros(max(n, 1), np.uint8)
    check(load().prx_mark_affected(ctx.handle, g.handle, int(mode), _p(du), _p(dv), len(du), _p(iu), len(iu),
                                   flags.ctypes.data), "prx_mark_affected")
    return flags[:n]


def _seed_csr(seed_sets):
    sets = [np.ascontiguousarray(x, dtype=np.uint32).ravel() for x in seed_sets]
    off = np.zeros(len(sets) + 1, np.uint32)
    off[1:] = np.cumsum([len(x) for x in sets])
    seeds = np.concatenate(sets) if sets else np.zeros(0, np.uint32)
    return off, np.ascontiguousarray(seeds, dtype=np.uint32)


def solve_ppr_batched(ctx, g, seed_sets, opts=None):
    """Personalized PageRank of len(seed_sets) teleport vectors (vector k
    teleports uniformly to seed_sets[k]) -> (ranks float64[n, nvec], result dict)."""
    n, _ = g.size()
    off, seeds = _seed_csr(seed_sets)
    nvec = len(off) - 1
    ranks = np.zeros((max(n, 1), max(nvec, 1)), np.float64)
    res = PprResult()
    check(load().prx_solve_ppr_batched(ctx.handle, g.handle, nvec, off.ctypes.data, _p(seeds),
                                       C.byref(opts or options()), ranks.ctypes.data, C.byref(res)),
          "prx_solve_ppr_batched")
    return ranks[:n, :nvec], res.as_dict()


def solve_ppr_batched_device(ctx, g, seed_sets, ranks_ptr, opts=None):
    """The same into device memory at ranks_ptr (n * nvec doubles) -> result dict."""
    off, seeds = _seed_csr(seed_sets)
    res = PprResult()
    check(load().prx_solve_ppr_batched_device(ctx.handle, g.handle, len(off) - 1, off.ctypes.data, _p(seeds),
                                              C.byref(opts or options()), ranks_ptr, C.byref(res)),
          "prx_solve_ppr_batched_device")
    return res.as_dict()


def autotune(ctx, g, cache_path=None):
    """Pick the MID / HIGH boundary and source-chunk widths for g by trial
    solves (prx_autotune) -> dict of the picks."""
    res = TuneResult()
    path = None if cache_path is None else str(cache_path).encode()
    check(load().prx_autotune(ctx.handle, g.handle, path, C.byref(res)), "prx_autotune")
    return res.as_dict()


def autotune_ppr(ctx, g):
    """Pick the batched personalized PageRank row split of g (warp-per-vertex
    bound, segment width) by trial solves (prx_autotune_ppr) -> dict."""
    from ._lib import PprTuneResult
    res = PprTuneResult()
    check(load().prx_autotune_ppr(ctx.handle, g.handle, C.byref(res)), "prx_autotune_ppr")
    return res.as_dict()


def selftest_division(ctx, dmax, per):
    """Mismatches of the solvers' reciprocal division against IEEE a / d."""
    bad = C.c_uint64(0)
    check(load().prx_selftest_division(ctx.handle, int(dmax), int(per), C.byref(bad)), "prx_selftest_division")
    return bad.value


# ---- the reference's five entry points ------------------------------------
def pagerank_static(ctx, g, opts=None):
    return solve(ctx, g, _lib.STATIC, opts=opts)


def pagerank_naive_dynamic(ctx, g, q, opts=None):
    return solve(ctx, g, _lib.NAIVE_DYNAMIC, q=q, opts=opts)


def pagerank_dynamic_traversal(ctx, g, deletions, insertions, q, opts=None):
    return solve(ctx, g, _lib.DYNAMIC_TRAVERSAL, deletions, insertions, q, opts)


def pagerank_dynamic_frontier(ctx, g, deletions, insertions, q, opts=None):
    return solve(ctx, g, _lib.DYNAMIC_FRONTIER, deletions, insertions, q, opts)


def pagerank_prune_dynamic_frontier(ctx, g, deletions, insertions, q, opts=None):
    return solve(ctx, g, _lib.PRUNE_DYNAMIC_FRONTIER, deletions, insertions, q, opts)
