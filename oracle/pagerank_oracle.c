/*
 * pagerank_oracle.c -- CPU oracle for the GB300 PageRank path.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py as the checker / the timed CPU baseline.  The
 * product (the CUDA library) never links or calls this file.
 *
 * Compile with -ffp-contract=off: every multiply-add below is written out
 * either as a separate multiply and add (the reference's x86 CPU code) or as
 * an explicit fma() (the reference's GPU code, where nvcc contracts
 * `C0 + P*c` into one DFMA).
 *
 * All citations are paths inside puzzlef/pagerank-cuda-dynamic.
 */
#include "pagerank_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* Contribution sum in the reference GPU order.                               */
/* ------------------------------------------------------------------------- */

/* Sum of r[u]/outdeg(u) over the in-edges of v, in the order the reference's
 * GPU kernels add them:
 *  - in-degree <= 64: one thread adds the terms front to back
 *    (pagerankUpdateRanksThreadCukU, inc/pagerankCuda.hxx:87-109, with
 *    pagerankCalculateContribCud :32-43 at stride 1);
 *  - in-degree  > 64: 256 threads each add the terms t, t+256, ... front to
 *    back (pagerankCalculateContribCud at stride 256, :177), then the 256
 *    partial sums are folded by the halving tree of sumValuesBlockReduceCudU
 *    (inc/_cuda.hxx:541-551): a[i] += a[(N+1)/2 + i] for i < N/2.
 * Each term is r[u]/d with d the out-degree converted to double, exactly the
 * expression at inc/pagerankCuda.hxx:40. */
static double contrib_sum_gpu(const uint32_t* xtoff, const uint32_t* xtedg,
                              const uint32_t* xtdat, const double* r, uint32_t v) {
  uint64_t s = xtoff[v], d = (uint64_t)xtoff[v + 1] - s;
  if (d <= 64) {
    double a = 0.0;
    for (uint64_t i = 0; i < d; ++i) {
      uint32_t u = xtedg[s + i];
      a += r[u] / (double)xtdat[u];
    }
    return a;
  }
  double part[256];
  for (uint64_t t = 0; t < 256; ++t) {
    double a = 0.0;
    for (uint64_t i = t; i < d; i += 256) {
      uint32_t u = xtedg[s + i];
      a += r[u] / (double)xtdat[u];
    }
    part[t] = a;
  }
  for (uint64_t N = 256; N > 1;) {
    uint64_t DN = (N + 1) / 2;
    for (uint64_t i = 0; i < N / 2; ++i) part[i] += part[DN + i];
    N = DN;
  }
  return part[0];
}

/* ------------------------------------------------------------------------- */
/* Affected-vertex marking (integer work).                                    */
/* ------------------------------------------------------------------------- */

/* Mark vaff[w] for every out-neighbour w of each u with naff[u]
 * (pagerankAffectedExtendThreadCukU / ...BlockCukU, inc/pagerankCuda.hxx:313-366,
 * pagerankMarkNeighborsCudU :55-63). */
static void expand_marks(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                         const uint8_t* naff, uint8_t* vaff) {
  /* threads only store 1s, so the result is independent of their order */
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    if (!naff[u]) continue;
    for (uint64_t i = xoff[u]; i < xoff[u + 1]; ++i) {
      #pragma omp atomic write
      vaff[xedg[i]] = 1;
    }
  }
}

/* Seed flags from the batch (pagerankAffectedFrontierPartialCukU,
 * inc/pagerankCuda.hxx:272-281): deletion (u,v) -> naff[u], vaff[v];
 * insertion (u,.) -> naff[u]. */
static void seed_marks(const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                       const uint32_t* insu, uint64_t ni, uint8_t* naff, uint8_t* vaff) {
  for (uint64_t i = 0; i < nd; ++i) { naff[delu[i]] = 1; vaff[delv[i]] = 1; }
  for (uint64_t i = 0; i < ni; ++i) naff[insu[i]] = 1;
}

void orc_mark_frontier(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                       const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                       const uint32_t* insu, uint64_t ni, uint8_t* vaff) {
  /* pagerankAffectedFrontierCuW, inc/pagerankCuda.hxx:405-412 */
  uint8_t* naff = (uint8_t*)calloc(n ? n : 1, 1);
  memset(vaff, 0, n);
  seed_marks(delu, delv, nd, insu, ni, naff, vaff);
  expand_marks(n, xoff, xedg, naff, vaff);
  free(naff);
}

void orc_mark_traversal(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                        const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                        const uint32_t* insu, uint64_t ni, uint8_t* vaff) {
  /* pagerankAffectedTraversalCuW, inc/pagerankCuda.hxx:438-456: start from the
   * DF marking, then repeatedly expand the whole last expansion (naff <- buff)
   * and OR it into vaff until the count of vaff stops changing.  Level k's
   * expansion is the set of vertices k out-steps from the DF marking, and once
   * a level adds nothing every later level lies inside vaff too, so the loop
   * ends with every vertex reachable from the DF marking.  That set is formed
   * here by one breadth-first search (O(n + m) instead of a scan of all n
   * flags per level, which on a 4096 x 4096 grid means thousands of levels). */
  orc_mark_frontier(n, xoff, xedg, delu, delv, nd, insu, ni, vaff);
  uint32_t* queue = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  uint64_t head = 0, tail = 0;
  for (uint32_t v = 0; v < n; ++v)
    if (vaff[v]) queue[tail++] = v;
  while (head < tail) {
    const uint32_t u = queue[head++];
    for (uint64_t i = xoff[u]; i < xoff[u + 1]; ++i) {
      const uint32_t w = xedg[i];
      if (!vaff[w]) { vaff[w] = 1; queue[tail++] = w; }
    }
  }
  free(queue);
}

/* ------------------------------------------------------------------------- */
/* GPU-semantics solver.                                                      */
/* ------------------------------------------------------------------------- */

int orc_solve(int mode, uint32_t n, uint64_t m,
              const uint32_t* xoff, const uint32_t* xedg,
              const uint32_t* xtoff, const uint32_t* xtedg, const uint32_t* xtdat,
              const uint32_t* delu, const uint32_t* delv, uint64_t nd,
              const uint32_t* insu, const uint32_t* insv, uint64_t ni,
              const double* q, const orc_options* o,
              double* ranks, uint8_t* vaff_out) {
  (void)m; (void)insv;
  if (mode < ORC_STATIC || mode > ORC_PRUNE_DYNAMIC_FRONTIER || !o) return -1;
  if (n == 0) return 0;  /* empty graph: the reference returns {} (:869) */
  const int DYNAMIC  = mode >= ORC_DYNAMIC_TRAVERSAL;
  const int FRONTIER = mode >= ORC_DYNAMIC_FRONTIER;
  const int PRUNE    = mode == ORC_PRUNE_DYNAMIC_FRONTIER;
  const double P = o->damping, E = o->tolerance;
  const double D = o->frontier_tolerance, C = o->prune_tolerance;
  const int L = o->max_iterations;
  double* a = (double*)malloc(sizeof(double) * n);
  double* r = (double*)malloc(sizeof(double) * n);
  uint8_t* vaff = (uint8_t*)calloc(n, 1);
  uint8_t* naff = (uint8_t*)calloc(n, 1);
  /* Initial ranks: previous ranks if given, else 1/N
   * (inc/pagerankCuda.hxx:810,817-818, pagerankInitializeRanksCukW :232-239). */
  const int use_q = q && mode != ORC_STATIC;
  #pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; ++v) r[v] = a[v] = use_q ? q[v] : 1.0 / (double)n;
  /* Initial marking, only when the batch is non-empty (:927,956,985).  With an
   * empty batch the reference leaves vaff uninitialised; here it is all-zero. */
  if (DYNAMIC && (nd > 0 || ni > 0)) {
    if (FRONTIER) orc_mark_frontier(n, xoff, xedg, delu, delv, nd, insu, ni, vaff);
    else          orc_mark_traversal(n, xoff, xedg, delu, delv, nd, insu, ni, vaff);
  }
  if (vaff_out) memcpy(vaff_out, vaff, n);
  /* pagerankLoopCuU, inc/pagerankCuda.hxx:675-692. */
  const double C0 = (1 - P) / (double)n;  /* N = order, :679 */
  int l = 0;
  while (l < L) {
    if (FRONTIER) memset(naff, 0, n);
    /* vertices are independent within a sweep (each writes only its own
     * a[v], vaff[v], naff[v]), so threads do not change any result */
    #pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
      if (DYNAMIC && !vaff[v]) { a[v] = r[v]; continue; }
      const uint32_t d = xtdat[v];
      const double rv = r[v];
      const double cv = contrib_sum_gpu(xtoff, xtedg, xtdat, r, v);
      /* :102 / :182, with nvcc's contraction of C0 + P*x into one fma */
      const double av = PRUNE ? fma(P, cv - rv / (double)d, C0) * (1 / (1 - (P / (double)d)))
                              : fma(P, cv, C0);
      a[v] = av;
      const double ev = fabs(av - rv);
      if (FRONTIER && PRUNE && ev / fmax(rv, av) <= C) vaff[v] = 0;
      if (FRONTIER && ev / fmax(rv, av) > D) naff[v] = 1;
    }
    ++l;
    double el = 0.0;  /* liNormDeltaInplaceCuW, inc/_cuda.hxx:926-934 */
    #pragma omp parallel for schedule(static) reduction(max:el)
    for (int64_t v = 0; v < (int64_t)n; ++v) el = fmax(el, fabs(a[v] - r[v]));
    if (FRONTIER) expand_marks(n, xoff, xedg, naff, vaff);
    double* t = a; a = r; r = t;
    if (el < E) break;
  }
  memcpy(ranks, r, sizeof(double) * n);
  free(a); free(r); free(vaff); free(naff);
  return l;
}

/* ------------------------------------------------------------------------- */
/* Reference CPU solvers (the timed CPU baseline).                            */
/* ------------------------------------------------------------------------- */

int orc_cpu_static(uint32_t n, const uint32_t* xtoff, const uint32_t* xtedg,
                   const uint32_t* xtdat, const orc_options* o, double* ranks,
                   int threads, int sweeps_cap, double* time_ms) {
  /* pagerankStaticOmp<ASYNC=false> (inc/pagerank.hxx:474-482): init 1/N
   * (:303-313), then sync sweeps (pagerankUpdateRanksSyncOmp :217-227,
   * pagerankUpdateRank :131-141) and liNormDeltaOmp (inc/_vector.hxx:1266).
   * *time_ms (optional) covers what the reference's `time` covers
   * (:423-438): initialisation and sweeps, not the allocations. */
  if (time_ms) *time_ms = 0;
  if (n == 0) return 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  const double P = o->damping, E = o->tolerance;
  int L = o->max_iterations;
  if (sweeps_cap > 0 && sweeps_cap < L) L = sweeps_cap;
  double* a = (double*)malloc(sizeof(double) * n);
  double* r = (double*)malloc(sizeof(double) * n);
  const int64_t N = n;
#ifdef _OPENMP
  const double t0 = omp_get_wtime();
#endif
  #pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < N; ++v) { r[v] = 1.0 / (double)n; a[v] = r[v]; }
  const double C0 = (1 - P) / (double)n;
  int l = 0;
  for (l = 0; l < L;) {
    #pragma omp parallel for schedule(dynamic, 2048)
    for (int64_t v = 0; v < N; ++v) {
      double cv = 0.0;
      for (uint64_t i = xtoff[v]; i < xtoff[v + 1]; ++i) {
        uint32_t u = xtedg[i];
        cv += r[u] / (double)xtdat[u];
      }
      a[v] = C0 + P * cv;
    }
    ++l;
    double el = 0.0;
    #pragma omp parallel for schedule(static) reduction(max:el)
    for (int64_t v = 0; v < N; ++v) { double e = fabs(a[v] - r[v]); if (e > el) el = e; }
    double* t = a; a = r; r = t;
    if (el < E) break;
  }
#ifdef _OPENMP
  if (time_ms) *time_ms = (omp_get_wtime() - t0) * 1e3;
#endif
  memcpy(ranks, r, sizeof(double) * n);
  free(a); free(r);
  return l;
}

int orc_cpu_prune_dynamic_frontier(uint32_t n,
    const uint32_t* xoff_old, const uint32_t* xedg_old,
    const uint32_t* yoff, const uint32_t* yedg,
    const uint32_t* ytoff, const uint32_t* ytedg, const uint32_t* ytdat,
    const uint32_t* delu, uint64_t nd, const uint32_t* insu, uint64_t ni,
    const double* q, const orc_options* o, double* ranks, int threads) {
  /* pagerankPruneDynamicFrontierOmp<ASYNC=true> (inc/pagerankPrune.hxx:306-311):
   * r <- q (:343-352), mark x.out(del src) and y.out(ins src)
   * (inc/pagerank.hxx:663-676), then asynchronous sweeps
   * (pagerankPruneUpdateRanksAsyncOmp, inc/pagerankPrune.hxx:141-158) with
   * C0 = (1-P)/S (:247).  Asynchronous sweeps read ranks other threads are
   * writing, so results vary with the thread count; it is a timing baseline. */
  if (n == 0) return 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  const double P = o->damping, E = o->tolerance;
  const double D = o->frontier_tolerance, C = o->prune_tolerance;
  const int L = o->max_iterations;
  const int64_t N = n;
  double* r = (double*)malloc(sizeof(double) * n);
  uint8_t* vaff = (uint8_t*)calloc(n, 1);
  for (int64_t v = 0; v < N; ++v) r[v] = q[v];
  for (uint64_t i = 0; i < nd; ++i)
    for (uint64_t j = xoff_old[delu[i]]; j < xoff_old[delu[i] + 1]; ++j) vaff[xedg_old[j]] = 1;
  for (uint64_t i = 0; i < ni; ++i)
    for (uint64_t j = yoff[insu[i]]; j < yoff[insu[i] + 1]; ++j) vaff[yedg[j]] = 1;
  const double C0 = (1 - P) / (double)n;
  int l;
  for (l = 0; l < L;) {
    double el = 0.0;
    #pragma omp parallel for schedule(dynamic, 2048) reduction(max:el)
    for (int64_t u = 0; u < N; ++u) {
      if (!vaff[u]) continue;
      const double ru = r[u];
      double av = 0.0;
      for (uint64_t i = ytoff[u]; i < ytoff[u + 1]; ++i) {
        uint32_t w = ytedg[i];
        av += r[w] / (double)ytdat[w];
      }
      const uint32_t d = ytdat[u];
      const double au = (C0 + P * (av - ru / (double)d)) * (1 / (1 - (P / (double)d)));
      r[u] = au;
      const double eu = fabs(ru - au);
      if (eu > el) el = eu;
      if (eu / fmax(ru, au) <= C) vaff[u] = 0;
      if (eu / fmax(ru, au) <= D) continue;
      for (uint64_t i = yoff[u]; i < yoff[u + 1]; ++i) {
        uint32_t v = yedg[i];
        if (v != (uint32_t)u && !vaff[v]) vaff[v] = 1;
      }
    }
    ++l;
    if (el < E) break;
  }
  memcpy(ranks, r, sizeof(double) * n);
  free(r); free(vaff);
  return l;
}

/* ------------------------------------------------------------------------- */
/* Graph helpers.                                                             */
/* ------------------------------------------------------------------------- */

/* first index i in [0, cnt) with key[i] >= u (key ascending) */
static uint64_t lower_u32(const uint32_t* key, uint64_t cnt, uint32_t u) {
  uint64_t lo = 0, hi = cnt;
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if (key[mid] < u) lo = mid + 1; else hi = mid;
  }
  return lo;
}

/* Row u of the updated graph: the old row minus deleted targets, merged with
 * the inserted targets; writes it to out (when non-NULL), returns its length. */
static uint64_t apply_row(const uint32_t* xedg, uint64_t i, uint64_t e,
                          const uint32_t* delv, uint64_t id, uint64_t id_end,
                          const uint32_t* insv, uint64_t ii, uint64_t ii_end, uint32_t* out) {
  uint64_t k = 0;
  for (;;) {
    const int has_old = i < e;
    const int has_ins = ii < ii_end;
    if (!has_old && !has_ins) break;
    uint32_t w;
    if (has_old && (!has_ins || xedg[i] < insv[ii])) {
      w = xedg[i++];
      while (id < id_end && delv[id] < w) ++id;
      if (id < id_end && delv[id] == w) { ++id; continue; }
    } else if (has_old && has_ins && xedg[i] == insv[ii]) {
      w = xedg[i++]; ++ii;  /* insertion of an existing edge: kept once */
    } else {
      w = insv[ii++];
    }
    if (out) out[k] = w;
    ++k;
  }
  return k;
}

uint64_t orc_apply_batch(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                         const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                         const uint32_t* insu, const uint32_t* insv, uint64_t ni,
                         uint32_t* yoff, uint32_t* yedg, uint64_t m_cap) {
  /* applyBatchUpdateOmpU (inc/batch.hxx:239-247) on sorted adjacency
   * (LazyBitset keeps keys ascending): each row becomes
   * (old row minus deleted targets) merged with inserted targets.  The batch
   * is sorted by source, so each row finds its deletions and insertions by
   * binary search and rows are built independently: lengths, a scan, then
   * the rows themselves. */
  uint64_t* len = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)n + 1));
  if (!len) return UINT64_MAX;
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    const uint64_t d0 = lower_u32(delu, nd, (uint32_t)u), d1 = lower_u32(delu, nd, (uint32_t)u + 1);
    const uint64_t i0 = lower_u32(insu, ni, (uint32_t)u), i1 = lower_u32(insu, ni, (uint32_t)u + 1);
    len[u] = (d0 == d1 && i0 == i1) ? (uint64_t)xoff[u + 1] - xoff[u]
                                     : apply_row(xedg, xoff[u], xoff[u + 1], delv, d0, d1, insv, i0, i1, NULL);
  }
  uint64_t k = 0;
  for (uint32_t u = 0; u < n; ++u) {
    const uint64_t l = len[u];
    len[u] = k;
    k += l;
  }
  if (k > m_cap || k > 0xffffffffull) { free(len); return UINT64_MAX; }
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    const uint64_t d0 = lower_u32(delu, nd, (uint32_t)u), d1 = lower_u32(delu, nd, (uint32_t)u + 1);
    const uint64_t i0 = lower_u32(insu, ni, (uint32_t)u), i1 = lower_u32(insu, ni, (uint32_t)u + 1);
    yoff[u] = (uint32_t)len[u];
    if (d0 == d1 && i0 == i1)
      memcpy(yedg + len[u], xedg + xoff[u], sizeof(uint32_t) * ((uint64_t)xoff[u + 1] - xoff[u]));
    else
      apply_row(xedg, xoff[u], xoff[u + 1], delv, d0, d1, insv, i0, i1, yedg + len[u]);
  }
  yoff[n] = (uint32_t)k;
  free(len);
  return k;
}

void orc_transpose(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                   uint32_t* xtoff, uint32_t* xtedg, uint32_t* xtdat) {
  /* transposeWithDegreeOmp (inc/transpose.hxx:110-134): vertex value = the
   * out-degree in x; in-edge rows hold sources ascending. */
  memset(xtoff, 0, sizeof(uint32_t) * ((size_t)n + 1));
  for (uint32_t u = 0; u < n; ++u) {
    xtdat[u] = xoff[u + 1] - xoff[u];
    for (uint64_t i = xoff[u]; i < xoff[u + 1]; ++i) xtoff[xedg[i] + 1]++;
  }
  for (uint32_t v = 0; v < n; ++v) xtoff[v + 1] += xtoff[v];
  uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  memcpy(fill, xtoff, sizeof(uint32_t) * n);
  for (uint32_t u = 0; u < n; ++u)
    for (uint64_t i = xoff[u]; i < xoff[u + 1]; ++i) xtedg[fill[xedg[i]]++] = u;
  free(fill);
}
