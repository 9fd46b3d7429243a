"""The reference driver's experiment, on the device (main.cu:48-171).

    python -m pagerank_gb300.experiment <file> <rows> <size> <unused> <batch_fraction>
           [--batches B] [--repeat R] [--partition] [--precision fp64|fp32] [--device D]

Same arguments as the reference's a.out (main.cu:158-161; the fourth is not
read there either).  The graph is the first 90% of the lines of a SNAP
temporal file plus a self-loop on every vertex; each of B batches inserts the
next batch_fraction * size lines (tidied against the current graph) and the
batches accumulate (main.cu:143-144).  Per batch the five CUDA techniques
run in main.cu's order (Static, Naive-dynamic, Dynamic Frontier, Dynamic
Frontier with Pruning, Dynamic Traversal), each dynamic one warm-started
from its own previous result, and print main.cu's result line with the L1
error against a Static solve run to tolerance 1e-100 (the reference computes
that one on the CPU, main.cu:88).  The OpenMP techniques of main.cu are CPU
code and are not run; --partition adds the ...CudaPartition lines (the
reference's PARTITION=true template, which gives the same ranks here).
Reading, ingest, tidy and apply all run through the library: the file is
parsed on the host, the graph is built and updated on the device.
"""
import argparse
import sys
import time

import numpy as np

from . import _lib
from .api import Context, Graph, options, solve
from .graphs import EdgeReader
from .report import glog_line

TECHNIQUES = (("pagerankStaticCuda", _lib.STATIC), ("pagerankNaiveDynamicCuda", _lib.NAIVE_DYNAMIC),
              ("pagerankDynamicFrontierCuda", _lib.DYNAMIC_FRONTIER),
              ("pagerankPruneDynamicFrontierCuda", _lib.PRUNE_DYNAMIC_FRONTIER),
              ("pagerankDynamicTraversalCuda", _lib.DYNAMIC_TRAVERSAL))


def _stamp():
    return time.strftime("%Y-%m-%d %H:%M:%S")


def run(path, rows, size, batch_fraction, batches=100, repeat=1, partition=False, precision="fp64", device=0,
        out=None):
    """Run the experiment; lines go to out (a callable, default print).
    Returns the result lines."""
    lines = []

    def emit(s, stamp=False):
        s = f"{_stamp()} {s}" if stamp else s   # LOG(...) of inc/_debug.hxx:193
        lines.append(s)
        (out or print)(s)

    ctx = Context(device)
    sms = _sm_count(device)
    emit(f"OMP_NUM_THREADS={sms}", stamp=True)
    emit(f"Loading graph {path} ...", stamp=True)
    prec = _lib.FP32_REFINE if precision == "fp32" else _lib.FP64
    run_opts = [options(repeat=repeat, precision=prec, partition=p) for p in ((0, 1) if partition else (0,))]
    exact = options(tolerance=1e-100)
    with EdgeReader(path) as reader:
        u, v, _ = reader.next(rows, int(0.90 * size))
        g0 = Graph.from_edges(ctx, rows, u, v, self_loops=False)
        emit(f"order: {rows} size: {g0.size()[1]} [directed] {{}} (90%)", stamp=True)
        g0.close()
        g = Graph.from_edges(ctx, rows, u, v, self_loops=True)
        m = g.size()[1]
        emit(f"order: {rows} size: {m} [directed] {{}} (selfLoopAllVertices)", stamp=True)
        emit(f"order: {rows} size: {m} [directed] {{}} (transposeWithDegree)", stamp=True)
        r0, _ = solve(ctx, g, _lib.STATIC, opts=exact)
        prev = {(t, p): r0 for t, _ in TECHNIQUES[1:] for p in range(len(run_opts))}
        empty = np.zeros(0, np.uint32)
        for b in range(batches):
            bu, bv, _ = reader.next(rows, int(batch_fraction * size))
            du, dv, iu, iv = g.tidy_batch(empty, empty, bu, bv)
            g.apply_batch(du, dv, iu, iv)
            emit(f"order: {rows} size: {g.size()[1]} [directed] {{}} (insertions={len(iu)})", stamp=True)
            s0, _ = solve(ctx, g, _lib.STATIC, opts=exact)
            for tech, mode in TECHNIQUES:
                for p, o in enumerate(run_opts):
                    q = prev.get((tech, p))
                    r, res = solve(ctx, g, mode, (du, dv), (iu, iv), q, o)
                    err = float(np.abs(r - s0).sum())
                    name = tech + ("Partition" if p else "")
                    emit(glog_line(res, name, err, b, sms, 0.0, batch_fraction))
                    if q is not None:
                        prev[(tech, p)] = r
        g.close()
    ctx.close()
    return lines


def _sm_count(device):
    import torch
    return torch.cuda.get_device_properties(device).multi_processor_count


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("file")
    p.add_argument("rows", type=int)
    p.add_argument("size", type=int)
    p.add_argument("unused", nargs="?", default="0")
    p.add_argument("batch_fraction", type=float, nargs="?", default=1e-4)
    p.add_argument("--batches", type=int, default=100)
    p.add_argument("--repeat", type=int, default=1)
    p.add_argument("--partition", action="store_true")
    p.add_argument("--precision", default="fp64", choices=("fp64", "fp32"))
    p.add_argument("--device", type=int, default=0)
    a = p.parse_args(argv)
    run(a.file, a.rows, a.size, a.batch_fraction, a.batches, a.repeat, a.partition, a.precision, a.device,
        out=lambda s: print(s, flush=True))


if __name__ == "__main__":
    sys.exit(main())
