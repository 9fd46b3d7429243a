"""ctypes binding of oracle/liboracle.so (test infrastructure only).

The C restatement lives in oracle/pagerank_oracle.c; this module only builds
it (``make -C oracle``) and marshals numpy arrays.  Used by tests/ as the
checker and by bench.py as the CPU baseline; the product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

STATIC, NAIVE_DYNAMIC, DYNAMIC_TRAVERSAL, DYNAMIC_FRONTIER, PRUNE_DYNAMIC_FRONTIER = range(5)
MODE_NAMES = {
    "static": STATIC, "naive_dynamic": NAIVE_DYNAMIC, "dynamic_traversal": DYNAMIC_TRAVERSAL,
    "dynamic_frontier": DYNAMIC_FRONTIER, "prune_dynamic_frontier": PRUNE_DYNAMIC_FRONTIER,
}


class Options(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("frontier_tolerance", C.c_double),
                ("prune_tolerance", C.c_double), ("damping", C.c_double),
                ("max_iterations", C.c_int)]


def build(force=False):
    srcs = ("pagerank_oracle.c", "oracle_gen.c", "pagerank_oracle.h")
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, f)) for f in srcs):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        u32p, u8p, f64p = (np.ctypeslib.ndpointer(t, flags="C") for t in (np.uint32, np.uint8, np.float64))
        u64 = C.c_uint64
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = [C.c_int, C.c_uint32, u64, C.c_void_p, C.c_void_p, u32p, u32p, u32p,
                                C.c_void_p, C.c_void_p, u64, C.c_void_p, C.c_void_p, u64,
                                C.c_void_p, C.POINTER(Options), f64p, C.c_void_p]
        for f in (L.orc_mark_frontier, L.orc_mark_traversal):
            f.restype = None
            f.argtypes = [C.c_uint32, u32p, u32p, C.c_void_p, C.c_void_p, u64, C.c_void_p, u64, u8p]
        L.orc_cpu_static.restype = C.c_int
        L.orc_cpu_static.argtypes = [C.c_uint32, u32p, u32p, u32p, C.POINTER(Options), f64p, C.c_int, C.c_int,
                                     C.POINTER(C.c_double)]
        L.orc_cpu_prune_dynamic_frontier.restype = C.c_int
        L.orc_cpu_prune_dynamic_frontier.argtypes = [C.c_uint32, u32p, u32p, u32p, u32p, u32p, u32p, u32p,
                                                     C.c_void_p, u64, C.c_void_p, u64, f64p,
                                                     C.POINTER(Options), f64p, C.c_int]
        L.orc_apply_batch.restype = u64
        L.orc_apply_batch.argtypes = [C.c_uint32, u32p, u32p, C.c_void_p, C.c_void_p, u64,
                                      C.c_void_p, C.c_void_p, u64, u32p, u32p, u64]
        L.orc_transpose.restype = None
        L.orc_transpose.argtypes = [C.c_uint32, u32p, u32p, u32p, u32p, u32p]
        L.orc_transpose_omp.restype = None
        L.orc_transpose_omp.argtypes = [C.c_uint32, u32p, u32p, u32p, u32p, u32p]
        L.orc_gen_weblike.restype = C.c_int
        L.orc_gen_weblike.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_uint32, C.c_double, C.c_uint32,
                                      C.c_uint64, C.POINTER(C.POINTER(C.c_uint32)),
                                      C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.c_uint64)]
        L.orc_free.restype = None
        L.orc_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def options(tolerance=1e-10, frontier_tolerance=1e-6, prune_tolerance=1e-6, damping=0.85,
            max_iterations=500):
    return Options(tolerance, frontier_tolerance, prune_tolerance, damping, max_iterations)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _ptr(a):
    return None if a is None or len(a) == 0 else a.ctypes.data


def solve(mode, xoff, xedg, xtoff, xtedg, xtdat, delu=None, delv=None, insu=None, insv=None,
          q=None, opts=None, want_flags=False):
    """GPU-semantics solve; returns (ranks, iterations[, vaff])."""
    mode = MODE_NAMES.get(mode, mode)
    xtoff, xtedg, xtdat = _u32(xtoff), _u32(xtedg), _u32(xtdat)
    n = len(xtoff) - 1
    xoff = None if xoff is None else _u32(xoff)
    xedg = None if xedg is None else _u32(xedg)
    delu, delv, insu, insv = (None if a is None else _u32(a) for a in (delu, delv, insu, insv))
    nd = 0 if delu is None else len(delu)
    ni = 0 if insu is None else len(insu)
    qq = None if q is None else np.ascontiguousarray(q, dtype=np.float64)
    ranks = np.zeros(n, np.float64)
    flags = np.zeros(max(n, 1), np.uint8) if want_flags else None
    it = lib().orc_solve(mode, n, len(xtedg), _ptr(xoff), _ptr(xedg), xtoff, xtedg, xtdat,
                         _ptr(delu), _ptr(delv), nd, _ptr(insu), _ptr(insv), ni,
                         _ptr(qq), C.byref(opts or options()), ranks,
                         None if flags is None else flags.ctypes.data)
    if it < 0:
        raise ValueError("oracle rejected the arguments")
    return (ranks, it, flags[:n]) if want_flags else (ranks, it)


def mark(kind, xoff, xedg, delu, delv, insu):
    xoff, xedg, delu, delv, insu = (_u32(a) for a in (xoff, xedg, delu, delv, insu))
    n = len(xoff) - 1
    flags = np.zeros(max(n, 1), np.uint8)
    f = lib().orc_mark_frontier if kind == "frontier" else lib().orc_mark_traversal
    f(n, xoff, xedg, _ptr(delu), _ptr(delv), len(delu), _ptr(insu), len(insu), flags)
    return flags[:n]


def cpu_static(xtoff, xtedg, xtdat, opts=None, threads=0, sweeps_cap=0, with_time=False):
    """Reference CPU Static (sync, OpenMP) -> (ranks, iterations[, time_ms])."""
    xtoff, xtedg, xtdat = _u32(xtoff), _u32(xtedg), _u32(xtdat)
    n = len(xtoff) - 1
    ranks = np.zeros(n, np.float64)
    t = C.c_double()
    it = lib().orc_cpu_static(n, xtoff, xtedg, xtdat, C.byref(opts or options()), ranks, threads, sweeps_cap,
                              C.byref(t))
    return (ranks, it, t.value) if with_time else (ranks, it)


def cpu_prune_dynamic_frontier(xoff_old, xedg_old, yoff, yedg, ytoff, ytedg, ytdat, delu, insu, q,
                               opts=None, threads=0):
    arrs = [_u32(a) for a in (xoff_old, xedg_old, yoff, yedg, ytoff, ytedg, ytdat)]
    delu, insu = _u32(delu), _u32(insu)
    n = len(arrs[0]) - 1
    ranks = np.zeros(n, np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    it = lib().orc_cpu_prune_dynamic_frontier(n, *arrs, _ptr(delu), len(delu), _ptr(insu), len(insu), q,
                                              C.byref(opts or options()), ranks, threads)
    return ranks, it


def apply_batch(xoff, xedg, delu, delv, insu, insv):
    xoff, xedg, delu, delv, insu, insv = (_u32(a) for a in (xoff, xedg, delu, delv, insu, insv))
    n = len(xoff) - 1
    cap = len(xedg) + len(insu)
    yoff = np.zeros(n + 1, np.uint32)
    yedg = np.empty(max(cap, 1), np.uint32)
    k = lib().orc_apply_batch(n, xoff, xedg, _ptr(delu), _ptr(delv), len(delu), _ptr(insu), _ptr(insv),
                              len(insu), yoff, yedg, cap)
    if k == 2 ** 64 - 1:
        raise ValueError("capacity exceeded")
    return yoff, yedg[:k]


def transpose(xoff, xedg, threads=False):
    """(xtoff, xtedg, xtdat) of an out-CSR; threads=True runs the OpenMP
    version (same output)."""
    xoff, xedg = _u32(xoff), _u32(xedg)
    n = len(xoff) - 1
    xtoff = np.zeros(n + 1, np.uint32)
    xtedg = np.empty(max(len(xedg), 1), np.uint32)
    xtdat = np.zeros(max(n, 1), np.uint32)
    (lib().orc_transpose_omp if threads else lib().orc_transpose)(n, xoff, xedg, xtoff, xtedg, xtdat)
    return xtoff, xtedg[:len(xedg)], xtdat[:n]


def _take(ptr, count):
    """Copy `count` uint32 from a malloc'd oracle array into numpy and free it."""
    try:
        return np.ctypeslib.as_array(ptr, shape=(count,)).copy() if count else np.zeros(0, np.uint32)
    finally:
        lib().orc_free(ptr)


def gen_weblike(n, alpha=2.1, dmin=5.9, dmax=100000, local=0.7, window=4096, seed=42):
    """The web-like generator's graph (the product's host generator gives
    the same arrays) -> (xoff, xedg)."""
    po, pe = C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)()
    m = C.c_uint64()
    st = lib().orc_gen_weblike(n, alpha, dmin, dmax, local, window, seed, C.byref(po), C.byref(pe), C.byref(m))
    if st != 0:
        raise ValueError(f"orc_gen_weblike failed ({st})")
    return _take(po, n + 1), _take(pe, m.value)
