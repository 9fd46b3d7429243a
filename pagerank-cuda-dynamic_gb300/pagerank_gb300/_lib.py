"""ctypes binding of libpagerank_gb300.so (the C ABI in include/pagerank_gb300.h).

This is the reference-side binding a Python caller would add: one ctypes
declaration per exported entry point.  Loading fails loudly when the library
is missing -- there is no fallback implementation.
"""
import ctypes as C
import os

from . import build as _build

STATIC, NAIVE_DYNAMIC, DYNAMIC_TRAVERSAL, DYNAMIC_FRONTIER, PRUNE_DYNAMIC_FRONTIER = range(5)
FP64, FP32_REFINE = 0, 1
LOOP_AUTO, LOOP_HOST, LOOP_GRAPH = 0, 1, 2

STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "device wait timed out",
          5: "size out of range", 6: "invalid state", 7: "did not converge"}


class Options(C.Structure):
    """prx_options (PagerankOptions<V>, inc/pagerank.hxx:24-55, plus GB300 knobs)."""
    _fields_ = [("repeat", C.c_int), ("tolerance", C.c_double), ("frontier_tolerance", C.c_double),
                ("prune_tolerance", C.c_double), ("damping", C.c_double), ("max_iterations", C.c_int),
                ("precision", C.c_int), ("loop", C.c_int), ("partition", C.c_int), ("timing", C.c_int),
                ("expansion", C.c_int), ("chunk_vertices", C.c_uint32), ("refine_sweeps", C.c_int),
                ("l2_fetch_bytes", C.c_int), ("require_convergence", C.c_int),
                ("hot_sources", C.c_int), ("int_adds", C.c_int)]


class Result(C.Structure):
    """prx_result (PagerankResult<V>, inc/pagerank.hxx:64-113, minus the ranks)."""
    _fields_ = [("iterations", C.c_int), ("time_ms", C.c_float), ("initialization_time_ms", C.c_float),
                ("marking_time_ms", C.c_float), ("computation_time_ms", C.c_float),
                ("affected_initial", C.c_uint64), ("edges_processed", C.c_uint64),
                ("last_delta", C.c_double), ("refinements", C.c_int), ("kernel_launches", C.c_uint64),
                ("update_ms", C.c_double * 3), ("update_launches", C.c_uint32 * 3),
                ("update32_ms", C.c_double * 3), ("update32_launches", C.c_uint32 * 3)]

    def as_dict(self):
        d = {}
        for k, _ in self._fields_:
            v = getattr(self, k)
            d[k] = list(v) if hasattr(v, "__len__") else v
        return d


class PprResult(C.Structure):
    """prx_ppr_result (batched personalized PageRank; no counterpart in the reference)."""
    _fields_ = [("iterations", C.c_int), ("fp64_sweeps", C.c_int), ("fp32_sweeps", C.c_int),
                ("refinements", C.c_int), ("time_ms", C.c_float), ("last_delta", C.c_double),
                ("kernel_launches", C.c_uint64), ("graph_launches", C.c_uint64), ("low_max", C.c_uint32),
                ("seg_edges", C.c_uint32)]

    as_dict = Result.as_dict


class PprTuneResult(C.Structure):
    """prx_ppr_tune_result (personalized PageRank thresholds; no counterpart in the reference)."""
    _fields_ = [("low_max", C.c_uint32), ("seg_edges", C.c_uint32), ("ms_per_solve", C.c_float),
                ("trials", C.c_int)]

    as_dict = Result.as_dict


class TuneResult(C.Structure):
    """prx_tune_result (autotuner picks; no counterpart in the reference)."""
    _fields_ = [("mid_max", C.c_uint32), ("chunk_vertices64", C.c_uint32), ("chunk_vertices32", C.c_uint32),
                ("ms_per_iteration64", C.c_float), ("ms_per_iteration32", C.c_float), ("trials", C.c_int),
                ("cached", C.c_int), ("l2_fetch_bytes", C.c_int), ("int_adds", C.c_int)]

    as_dict = Result.as_dict


class HostCsr(C.Structure):
    _fields_ = [("n", C.c_uint32), ("m", C.c_uint64), ("off", C.POINTER(C.c_uint32)),
                ("edg", C.POINTER(C.c_uint32))]


class PrxError(RuntimeError):
    def __init__(self, status, where, detail=""):
        super().__init__(f"{where}: {STATUS.get(status, status)}" + (f" ({detail})" if detail else ""))
        self.status = status


_lib = None
EXPORTS = (
    "prx_options_default", "prx_status_string", "prx_last_error", "prx_context_create", "prx_context_destroy",
    "prx_context_stream", "prx_graph_create", "prx_graph_create64", "prx_graph_download64", "prx_graph_destroy",
    "prx_release_cached_memory", "prx_graph_pool_stats", "prx_l2_fetch_granularity", "prx_graph_size",
    "prx_graph_class_stats",
    "prx_graph_download",
    "prx_graph_apply_batch", "prx_solve", "prx_solve_device", "prx_solve_batches_device", "prx_mark_affected",
    "prx_selftest_division",
    "prx_solve_ppr_batched", "prx_solve_ppr_batched_device", "prx_graph_set_weights", "prx_solve_weighted",
    "prx_adjoint", "prx_autotune", "prx_autotune_ppr", "prx_graph_tidy_batch", "prx_graph_create_from_edges",
    "prx_graph_create_from_edges_device", "prx_graph_gen_batch",
    "prx_edge_reader_open", "prx_edge_reader_next", "prx_edge_reader_close", "prx_read_mtx", "prx_format_glog",
    "prx_graph_create_from_text", "prx_edge_reader_next_graph", "prx_graph_create_from_mtx", "prx_format_edges",
    "prx_host_csr_free",
    "prx_gen_rmat", "prx_gen_weblike", "prx_gen_grid", "prx_gen_batch", "prx_host_tidy_batch",
    "prx_host_apply_batch", "prx_host_transpose", "prx_host_free",
)


def library_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Load the shared library (building it first if asked and absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libpagerank_gb300.so not built ({path}); run __graft_entry__.build()")
        _build.build()
    L = C.CDLL(path)
    vp, u32p, u64, i32, dbl = C.c_void_p, C.POINTER(C.c_uint32), C.c_uint64, C.c_int, C.c_double
    sig = {
        "prx_options_default": (None, [C.POINTER(Options)]),
        "prx_status_string": (C.c_char_p, [i32]),
        "prx_last_error": (C.c_char_p, []),
        "prx_context_create": (i32, [i32, C.POINTER(vp)]),
        "prx_context_destroy": (i32, [vp]),
        "prx_context_stream": (vp, [vp]),
        "prx_graph_create": (i32, [vp, C.c_uint32, u64, vp, vp, vp, vp, vp, i32, C.POINTER(vp)]),
        "prx_graph_create64": (i32, [vp, C.c_uint32, u64, vp, vp, vp, vp, vp, i32, C.c_uint32, C.POINTER(vp)]),
        "prx_graph_download64": (i32, [vp, vp, vp, vp, vp, vp]),
        "prx_graph_destroy": (i32, [vp]),
        "prx_release_cached_memory": (i32, [i32]),
        "prx_l2_fetch_granularity": (i32, [i32, i32, C.POINTER(i32)]),
        "prx_graph_pool_stats": (i32, [i32, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
        "prx_graph_size": (i32, [vp, C.POINTER(C.c_uint32), C.POINTER(u64)]),
        "prx_graph_class_stats": (i32, [vp, C.POINTER(C.c_uint32), C.POINTER(u64)]),
        "prx_graph_download": (i32, [vp, vp, vp, vp, vp, vp]),
        "prx_graph_apply_batch": (i32, [vp, vp, vp, u64, vp, vp, u64]),
        "prx_solve": (i32, [vp, vp, i32, vp, vp, u64, vp, vp, u64, vp, C.POINTER(Options), vp, C.POINTER(Result)]),
        "prx_solve_device": (i32, [vp, vp, i32, vp, vp, u64, vp, vp, u64, vp, C.POINTER(Options), vp,
                                   C.POINTER(Result)]),
        "prx_solve_batches_device": (i32, [vp, vp, i32, C.c_uint32, vp, vp, vp, vp, vp, vp, vp, C.POINTER(Options),
                                           vp, vp, vp, C.POINTER(C.c_uint32)]),
        "prx_mark_affected": (i32, [vp, vp, i32, vp, vp, u64, vp, u64, vp]),
        "prx_selftest_division": (i32, [vp, C.c_uint32, C.c_uint32, C.POINTER(u64)]),
        "prx_solve_ppr_batched": (i32, [vp, vp, C.c_uint32, vp, vp, C.POINTER(Options), vp, C.POINTER(PprResult)]),
        "prx_solve_ppr_batched_device": (i32, [vp, vp, C.c_uint32, vp, vp, C.POINTER(Options), vp,
                                               C.POINTER(PprResult)]),
        "prx_graph_set_weights": (i32, [vp, vp, vp]),
        "prx_autotune": (i32, [vp, vp, C.c_char_p, C.POINTER(TuneResult)]),
        "prx_autotune_ppr": (i32, [vp, vp, C.POINTER(PprTuneResult)]),
        "prx_graph_tidy_batch": (i32, [vp, vp, vp, vp, u64, vp, vp, u64, vp, vp, C.POINTER(u64), vp, vp,
                                       C.POINTER(u64)]),
        "prx_graph_create_from_edges": (i32, [vp, C.c_uint32, vp, vp, u64, i32, C.POINTER(vp)]),
        "prx_graph_create_from_edges_device": (i32, [vp, C.c_uint32, vp, vp, u64, i32, C.POINTER(vp)]),
        "prx_graph_gen_batch": (i32, [vp, vp, u64, u64, u64, vp, vp, C.POINTER(u64), vp, vp, C.POINTER(u64)]),
        "prx_edge_reader_open": (i32, [C.c_char_p, C.POINTER(vp)]),
        "prx_edge_reader_next": (i32, [vp, C.c_uint32, u64, i32, C.POINTER(u32p), C.POINTER(u32p), C.POINTER(u64),
                                       C.POINTER(u64)]),
        "prx_edge_reader_close": (i32, [vp]),
        "prx_graph_create_from_text": (i32, [vp, C.c_char_p, u64, C.c_uint32, u64, i32, i32, C.POINTER(vp),
                                             C.POINTER(u64), C.POINTER(u64)]),
        "prx_edge_reader_next_graph": (i32, [vp, vp, C.c_uint32, u64, i32, i32, C.POINTER(vp), C.POINTER(u64)]),
        "prx_format_edges": (i32, [vp, vp, u64, C.POINTER(C.c_void_p), C.POINTER(u64)]),
        "prx_graph_create_from_mtx": (i32, [vp, C.c_char_p, i32, C.POINTER(vp), C.POINTER(C.c_uint32)]),
        "prx_format_glog": (i32, [C.c_char_p, C.c_size_t, dbl, dbl, i32, i32, C.POINTER(Result), dbl, C.c_char_p]),
        "prx_read_mtx": (i32, [C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(u32p), C.POINTER(u32p),
                               C.POINTER(u64)]),
        "prx_solve_weighted": (i32, [vp, vp, vp, vp, C.POINTER(Options), vp, C.POINTER(Result)]),
        "prx_adjoint": (i32, [vp, vp, vp, vp, vp, C.POINTER(Options), vp, vp, vp, C.POINTER(dbl),
                              C.POINTER(Result)]),
        "prx_host_csr_free": (None, [C.POINTER(HostCsr)]),
        "prx_gen_rmat": (i32, [i32, i32, dbl, dbl, dbl, u64, C.POINTER(HostCsr)]),
        "prx_gen_weblike": (i32, [C.c_uint32, dbl, dbl, C.c_uint32, dbl, C.c_uint32, u64, C.POINTER(HostCsr)]),
        "prx_gen_grid": (i32, [C.c_uint32, dbl, u64, C.POINTER(HostCsr)]),
        "prx_gen_batch": (i32, [C.POINTER(HostCsr), u64, u64, u64, C.POINTER(u32p), C.POINTER(u32p),
                                C.POINTER(u64), C.POINTER(u32p), C.POINTER(u32p), C.POINTER(u64)]),
        "prx_host_tidy_batch": (i32, [C.POINTER(HostCsr), vp, vp, C.POINTER(u64), vp, vp, C.POINTER(u64)]),
        "prx_host_apply_batch": (i32, [C.POINTER(HostCsr), vp, vp, u64, vp, vp, u64, C.POINTER(HostCsr)]),
        "prx_host_transpose": (i32, [C.POINTER(HostCsr), C.POINTER(HostCsr), vp]),
        "prx_host_free": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status, where):
    if status != 0:
        detail = load().prx_last_error().decode(errors="replace")
        raise PrxError(status, where, detail)
