"""The bench's stdout line stays one short JSON record: every section is cut
down to a few scalars by summarize() and rounded by compact(), the full
sections going to the detail record (CPU test of the host-side helpers)."""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _sections():
    row = {"ms": 36.123456789, "iterations": 4, "marking_ms": 1.2345678, "affected_initial": 44104971,
           "edges": 7396812858, "touched_ge_s": 201.83206436, "speedup_vs_static": 1.44093615}
    dynamic = {"batches": [dict(size=s, static={"ms": 52.8, "iterations": 7}, nd=row, dt=row, df=row, dfp=row)
                           for s in (1e-5, 1e-4, 1e-3) for _ in range(10)],
               "median_speedup_vs_static": {str(s): {k: 1.23456789 for k in ("nd", "dt", "df", "dfp",
                                                                              "df_fp32_refine", "dfp_fp32_refine")}
                                            for s in (1e-05, 0.0001, 0.001)},
               "tidy": {"raw_edges": 2092169, "call_ms": 3.2488, "host_ms": 454.7, "same": True}}
    fp32 = {"ms_per_solve": 43.568123, "speedup_vs_fp64": 1.2416, "linf_vs_fp64": 1.2426e-14,
            "fp32_sweep_ms": 5.398, "fp32_low_gbs": 2937.1, "fp32_low_frac": 0.43247, "iterations": [7] * 10}
    dfp = {"dfp_ms": 36.67, "df_ms": 35.42, "static_ms": 52.75, "dfp_speedup_vs_static": 1.4386,
           "df_speedup_vs_static": 1.4894, "dfp_fp32_refine_ms": 27.98, "dfp_fp32_refine_speedup_vs_dfp_fp64": 1.31,
           "dfp_fp32_refine_speedup_vs_static": 1.8855, "dfp_fp32_refine_linf_vs_dfp_fp64": 1.365e-11,
           "cpu_dfp_ms": 5906.7, "cpu_dfp_iterations": 4, "cpu_dfp_threads": 16, "gpu_dfp_vs_cpu_dfp": 161.08,
           "batch": {"deletions": 38039, "insertions": 152158}}
    grid = {"static_ms": 5.8, "static_ge_s": 147.4, "dt": row, "df": row, "dfp": row}
    ppr = {"fp64": {"time_ms": 709.67}, "fp32_refine": {"time_ms": 220.09, "graph_launches": 1},
           "speedup_fp32_refine_vs_fp64": 3.2244, "fp32_refine_host_loop_ms": 220.17, "fp32_sweep_frac": 0.8197,
           "linf_fp32_refine_vs_fp64": 7.3766e-10}
    adj = {"fd_max_rel_err": 2.737e-09, "rounds": [{"fd_edges": 1000, "adjoint_ms": 52.3}] * 21}
    big = {"ge_s": 211.7, "copy_ranks_exactly_quarter_of_single": True, "ms": 359.4}
    ingest = {"device_ms": [244.3, 226.2]}
    tune = {"seconds": 1.104, "mid_max": 4096, "int_adds": 1}
    multi = {"batches": 10, "host_loop_ms": 866.79, "one_launch_ms": 590.37, "speedup_vs_host_loop": 1.4682,
             "graph_launches": 1, "same_bits": True, "step_ms": [58.0] * 10}
    return fp32, dfp, dynamic, grid, ppr, adj, big, ingest, tune, multi


def test_summary_is_short_and_scalar():
    s = bench.compact(bench.summarize(*_sections()))
    text = json.dumps(s)
    assert len(text) < 2500, len(text)   # the whole line stays under 4 KB with the headline keys
    assert json.loads(text) == s

    def leaves(x):
        if isinstance(x, dict):
            for v in x.values():
                yield from leaves(v)
        else:
            yield x
    assert all(not isinstance(v, list) for v in leaves(s))
    assert s["multibatch_dfp_1e-5_x10"]["same_bits"] is True
    assert s["adjoint_rmat20"]["fd_edges"] == 21000 and s["adjoint_rmat20"]["batches"] == 20


def test_compact_rounds_floats_only():
    x = {"a": 1.23456789, "b": [2.00000001, 3], "c": "text", "d": True, "e": 12345678}
    y = bench.compact(x, digits=4)
    assert y == {"a": 1.235, "b": [2.0, 3], "c": "text", "d": True, "e": 12345678}


def test_missing_sections_are_left_out():
    assert bench.summarize(None, None, None, None, None, None, None, None, None) == {}
