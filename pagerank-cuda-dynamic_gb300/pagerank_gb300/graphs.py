"""Host graph utilities of the C ABI: synthetic generators, batches, transpose,
edge-list readers (SNAP temporal text, MatrixMarket).

Arrays made by the library are wrapped without copying: the numpy array keeps
an owner object alive that frees the C buffer when the last view goes away.
"""
import ctypes as C

import numpy as np

from ._lib import HostCsr, check, load


class _Owned:
    """Numpy-visible view of a library-allocated uint32 buffer."""

    def __init__(self, ptr, count):
        self._addr = C.cast(ptr, C.c_void_p).value or 0
        self.__array_interface__ = {"shape": (int(count),), "typestr": "<u4", "version": 3,
                                    "data": (self._addr, False)}

    def __del__(self):
        if self._addr:
            load().prx_host_free(C.c_void_p(self._addr))
            self._addr = 0


def _take(ptr, count):
    if count == 0:
        load().prx_host_free(C.cast(ptr, C.c_void_p))
        return np.zeros(0, np.uint32)
    return np.asarray(_Owned(ptr, count))


def _take_csr(h):
    off = _take(h.off, h.n + 1)
    edg = _take(h.edg, h.m)
    return off, edg


def _as_csr(off, edg):
    off = np.ascontiguousarray(off, dtype=np.uint32)
    edg = np.ascontiguousarray(edg, dtype=np.uint32)
    h = HostCsr(len(off) - 1, len(edg), off.ctypes.data_as(C.POINTER(C.c_uint32)),
                edg.ctypes.data_as(C.POINTER(C.c_uint32)))
    return h, (off, edg)


def rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=42):
    """R-MAT, duplicates removed, self-loop on every vertex -> (off, edg)."""
    h = HostCsr()
    check(load().prx_gen_rmat(scale, edge_factor, a, b, c, seed, C.byref(h)), "prx_gen_rmat")
    return _take_csr(h)


def weblike(n, alpha=2.1, dmin=5.5, dmax=100000, local=0.7, window=4096, seed=42):
    """Web-like power-law graph (Zipf out-degree, id locality) -> (off, edg)."""
    h = HostCsr()
    check(load().prx_gen_weblike(n, alpha, dmin, dmax, local, window, seed, C.byref(h)), "prx_gen_weblike")
    return _take_csr(h)


def grid(w, diag=0.05, seed=42):
    """w x w grid, 4-neighbour both ways, diagonal shortcuts, self-loops -> (off, edg)."""
    h = HostCsr()
    check(load().prx_gen_grid(w, diag, seed, C.byref(h)), "prx_gen_grid")
    return _take_csr(h)


def transpose(off, edg):
    """In-CSR (sources ascending) and out-degrees -> (xtoff, xtedg, xtdat)."""
    x, keep = _as_csr(off, edg)
    n = x.n
    xtdat = np.zeros(max(n, 1), np.uint32)
    h = HostCsr()
    check(load().prx_host_transpose(C.byref(x), C.byref(h), xtdat.ctypes.data), "prx_host_transpose")
    del keep
    xtoff, xtedg = _take_csr(h)
    return xtoff, xtedg, xtdat[:n]


def random_batch(off, edg, n_del, n_ins, seed=7):
    """Random batch (uniform insertions, uniform existing non-self-loop
    deletions), tidied -> (del_u, del_v, ins_u, ins_v)."""
    x, keep = _as_csr(off, edg)
    P = C.POINTER(C.c_uint32)
    du, dv, iu, iv = P(), P(), P(), P()
    nd, ni = C.c_uint64(), C.c_uint64()
    check(load().prx_gen_batch(C.byref(x), n_del, n_ins, seed, C.byref(du), C.byref(dv), C.byref(nd),
                               C.byref(iu), C.byref(iv), C.byref(ni)), "prx_gen_batch")
    del keep
    return (_take(du, nd.value), _take(dv, nd.value), _take(iu, ni.value), _take(iv, ni.value))


def tidy_batch(off, edg, del_u, del_v, ins_u, ins_v):
    """tidyBatchUpdateU (inc/batch.hxx:200-208) -> tidied copies."""
    x, keep = _as_csr(off, edg)
    du, dv, iu, iv = (np.array(a, dtype=np.uint32, copy=True) for a in (del_u, del_v, ins_u, ins_v))
    nd, ni = C.c_uint64(len(du)), C.c_uint64(len(iu))
    check(load().prx_host_tidy_batch(C.byref(x), du.ctypes.data, dv.ctypes.data, C.byref(nd), iu.ctypes.data,
                                     iv.ctypes.data, C.byref(ni)), "prx_host_tidy_batch")
    del keep
    return du[:nd.value], dv[:nd.value], iu[:ni.value], iv[:ni.value]


def apply_batch(off, edg, del_u, del_v, ins_u, ins_v):
    """Out-CSR with a tidied batch applied (host) -> (off, edg)."""
    x, keep = _as_csr(off, edg)
    arrs = [np.ascontiguousarray(a, dtype=np.uint32) for a in (del_u, del_v, ins_u, ins_v)]
    h = HostCsr()
    check(load().prx_host_apply_batch(C.byref(x), arrs[0].ctypes.data, arrs[1].ctypes.data, len(arrs[0]),
                                      arrs[2].ctypes.data, arrs[3].ctypes.data, len(arrs[2]), C.byref(h)),
          "prx_host_apply_batch")
    del keep
    return _take_csr(h)


class EdgeReader:
    """SNAP temporal edge list read in consecutive pieces (prx_edge_reader_*),
    as the reference's driver reads its input (main.cu:167, main.cu:83)."""

    def __init__(self, path):
        self._h = C.c_void_p()
        check(load().prx_edge_reader_open(str(path).encode(), C.byref(self._h)), "prx_edge_reader_open")

    def next(self, rows, size, symmetric=False):
        """Next `size` lines -> (u, v, lines): 0-based ids, lines consumed."""
        u, v = C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)()
        cnt, lines = C.c_uint64(), C.c_uint64()
        check(load().prx_edge_reader_next(self._h, int(rows), int(size), int(bool(symmetric)), C.byref(u),
                                          C.byref(v), C.byref(cnt), C.byref(lines)), "prx_edge_reader_next")
        return _take(u, cnt.value), _take(v, cnt.value), lines.value

    def close(self):
        if self._h:
            load().prx_edge_reader_close(self._h)
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


def read_mtx(path):
    """MatrixMarket coordinate file -> (n, u, v), 0-based; symmetric files give both directions."""
    n = C.c_uint32()
    u, v = C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)()
    cnt = C.c_uint64()
    check(load().prx_read_mtx(str(path).encode(), C.byref(n), C.byref(u), C.byref(v), C.byref(cnt)), "prx_read_mtx")
    return n.value, _take(u, cnt.value), _take(v, cnt.value)


def format_edges(u, v):
    """prx_format_edges: "u v\\n" lines with 1-based ids -> bytes."""
    u = np.ascontiguousarray(u, dtype=np.uint32)
    v = np.ascontiguousarray(v, dtype=np.uint32)
    if len(u) != len(v):
        raise ValueError("u and v differ in length")
    ptr, n = C.c_void_p(), C.c_uint64()
    check(load().prx_format_edges(u.ctypes.data if len(u) else None, v.ctypes.data if len(v) else None, len(u),
                                  C.byref(ptr), C.byref(n)), "prx_format_edges")
    try:
        return (C.c_char * n.value).from_address(ptr.value).raw if n.value else b""
    finally:
        load().prx_host_free(ptr)
