/*
 * pagerank_oracle.h -- CPU oracle for the GB300 PageRank path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load this library, and
 * only as the checker or the timed CPU baseline -- never as the product path.
 *
 * The oracle restates, in plain C, the algorithms of puzzlef/pagerank-cuda-dynamic:
 *   - orc_solve():      the GPU solvers of inc/pagerankCuda.hxx (Static, ND, DT,
 *                       DF, DF-P) with the GPU's update rules, loop order and
 *                       summation order (see pagerank_oracle.c for file:line).
 *   - orc_mark_*():     the DF / DT affected-vertex marking (integer work).
 *   - orc_cpu_*():      the reference's OpenMP CPU solvers (inc/pagerank.hxx,
 *                       inc/pagerankPrune.hxx), used as the timed CPU baseline.
 *   - orc_apply_batch():the CSR effect of inc/batch.hxx applyBatchUpdateOmpU.
 *
 * Pinning: the restatement is checked against fixtures produced by the
 * reference's own CPU code (tests/golden/, made by tests/golden/make_golden.py
 * from oracle/ref_harness.cpp compiled against the reference headers).
 *
 * Graphs are dense CSR (vertex ids 0..n-1, the reference's vertexKeys order):
 *   xoff[n+1], xedg[m]   out-edges (targets ascending per row)
 *   xtoff[n+1], xtedg[m] in-edges  (sources ascending per row)
 *   xtdat[n]             out-degree of each vertex
 */
#ifndef PAGERANK_ORACLE_H
#define PAGERANK_ORACLE_H
#include <stdint.h>
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_STATIC = 0,
  ORC_NAIVE_DYNAMIC = 1,
  ORC_DYNAMIC_TRAVERSAL = 2,
  ORC_DYNAMIC_FRONTIER = 3,
  ORC_PRUNE_DYNAMIC_FRONTIER = 4
};

typedef struct {
  double tolerance;          /* E [1e-10] */
  double frontier_tolerance; /* D [1e-6]  */
  double prune_tolerance;    /* C [1e-6]  */
  double damping;            /* P [0.85]  */
  int    max_iterations;     /* L [500]   */
} orc_options;

/* GPU-semantics solve (inc/pagerankCuda.hxx:675-849).  ranks[n] receives the
 * final ranks; q may be NULL (start from 1/n).  vaff_out (optional, n bytes)
 * receives the affected flags after the initial marking.  Returns the number
 * of iterations, or -1 on bad arguments. */
int orc_solve(int mode, uint32_t n, uint64_t m,
              const uint32_t* xoff, const uint32_t* xedg,
              const uint32_t* xtoff, const uint32_t* xtedg, const uint32_t* xtdat,
              const uint32_t* delu, const uint32_t* delv, uint64_t nd,
              const uint32_t* insu, const uint32_t* insv, uint64_t ni,
              const double* q, const orc_options* o,
              double* ranks, uint8_t* vaff_out);

/* DF initial marking (inc/pagerankCuda.hxx:272-281, 313-366, 405-412). */
void orc_mark_frontier(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                       const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                       const uint32_t* insu, uint64_t ni, uint8_t* vaff);

/* DT marking: closure of the DF marking (inc/pagerankCuda.hxx:438-456). */
void orc_mark_traversal(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                        const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                        const uint32_t* insu, uint64_t ni, uint8_t* vaff);

/* Reference CPU Static PageRank, synchronous, OpenMP
 * (inc/pagerank.hxx:217-227, 413-440, 474-482).  Returns iterations; at
 * most sweeps_cap sweeps when sweeps_cap > 0; *time_ms (may be NULL) gets
 * the time of initialisation + sweeps, as the reference's `time`. */
int orc_cpu_static(uint32_t n, const uint32_t* xtoff, const uint32_t* xtedg,
                   const uint32_t* xtdat, const orc_options* o, double* ranks,
                   int threads, int sweeps_cap, double* time_ms);

/* Reference CPU DF-P, asynchronous, OpenMP (inc/pagerankPrune.hxx:141-158,
 * 227-263, 306-311), initial marking per inc/pagerank.hxx:663-676.  The
 * batch sources are needed for the marking; x is the graph before the batch.
 * Returns iterations. */
int orc_cpu_prune_dynamic_frontier(uint32_t n,
    const uint32_t* xoff_old, const uint32_t* xedg_old,
    const uint32_t* yoff, const uint32_t* yedg,
    const uint32_t* ytoff, const uint32_t* ytedg, const uint32_t* ytdat,
    const uint32_t* delu, uint64_t nd, const uint32_t* insu, uint64_t ni,
    const double* q, const orc_options* o, double* ranks, int threads);

/* Apply a tidied batch (sorted, unique, filtered by existence) to an out-CSR.
 * Writes the new offsets (n+1) and edges (capacity m_cap); returns the new
 * edge count, or UINT64_MAX if m_cap is too small. */
uint64_t orc_apply_batch(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                         const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                         const uint32_t* insu, const uint32_t* insv, uint64_t ni,
                         uint32_t* yoff, uint32_t* yedg, uint64_t m_cap);

/* Transpose an out-CSR into an in-CSR (sources ascending) and out-degrees. */
void orc_transpose(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                   uint32_t* xtoff, uint32_t* xtedg, uint32_t* xtdat);

/* Seeded synthetic inputs (oracle_gen.c): the product generators' graphs,
 * built without the product library.  orc_gen_weblike returns 0 and
 * malloc'd *xoff_out[n+1], *xedg_out[*m_out] (free with orc_free); -1 bad
 * arguments, -2 out of memory, -3 more than 2^32 - 1 edges. */
int orc_gen_weblike(uint32_t n, double alpha, double dmin, uint32_t dmax, double local,
                    uint32_t window, uint64_t seed, uint32_t** xoff_out, uint32_t** xedg_out,
                    uint64_t* m_out);
/* orc_transpose with OpenMP threads (same output). */
void orc_transpose_omp(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                       uint32_t* xtoff, uint32_t* xtedg, uint32_t* xtdat);
void orc_free(void* p);

#ifdef __cplusplus
}
#endif
#endif
