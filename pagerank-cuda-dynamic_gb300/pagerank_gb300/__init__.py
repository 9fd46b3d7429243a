"""GB300-native PageRank (Static, ND, DT, DF, DF-P) behind a C ABI.

The compute path is libpagerank_gb300.so (hand-written sm_103a kernels plus
host C++); this package only builds and binds it.
"""
from ._lib import (DYNAMIC_FRONTIER, DYNAMIC_TRAVERSAL, FP32_REFINE, FP64, LOOP_AUTO, LOOP_GRAPH, LOOP_HOST,
                   NAIVE_DYNAMIC, PRUNE_DYNAMIC_FRONTIER, STATIC, PrxError, library_path, load)
from .api import (Context, Graph, mark_affected, options, pagerank_dynamic_frontier, pagerank_dynamic_traversal,
                  pagerank_naive_dynamic, pagerank_prune_dynamic_frontier, pagerank_static, release_cached_memory,
                  l2_fetch_granularity, graph_pool_stats, selftest_division, solve, autotune, autotune_ppr,
                  solve_device, solve_batches, solve_ppr_batched, solve_ppr_batched_device)
from . import graphs

MODES = {"static": STATIC, "naive_dynamic": NAIVE_DYNAMIC, "dynamic_traversal": DYNAMIC_TRAVERSAL,
         "dynamic_frontier": DYNAMIC_FRONTIER, "prune_dynamic_frontier": PRUNE_DYNAMIC_FRONTIER}
