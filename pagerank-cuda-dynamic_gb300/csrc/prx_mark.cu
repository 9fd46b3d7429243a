// prx_mark.cu -- affected-vertex marking for DT / DF / DF-P (integer work).
//
// The reference keeps one byte flag per vertex and rescans all N flags in
// every kernel (inc/pagerankCuda.hxx:272-456, 681-687).  Here the affected
// set is a bitmap (N/8 bytes, resident in L2 for every graph size used) plus
// compact per-class lists of the affected vertices, so each iteration costs
// work proportional to the affected set, not to N.  A vertex enters a list
// exactly once per iteration: test_and_set() on the bitmap decides who
// appends it.  The resulting SET of affected vertices is the reference's:
//   seed:   deletion (u,v) -> expand u, mark v;  insertion (u,.) -> expand u
//           (pagerankAffectedFrontierPartialCukU :272-281)
//   expand: mark every out-neighbour of a vertex to expand
//           (pagerankAffectedExtend*CukU :313-366)
//   DT:     close the DF marking under out-edges (pagerankAffectedTraversalCuW
//           :438-456; the reference iterates until the count stops growing,
//           a breadth-first closure over newly marked vertices gives the
//           same set)
//   DF/DF-P per iteration: a vertex with relative change > D expands, one
//           with relative change <= C (DF-P) leaves the set (:106-107, 686-687).
#include "prx_device.cuh"

namespace prx {

// Deletion (u,v): u to the expand list, v affected.  Insertion (u,.): u to the
// expand list.  Expanded sources are deduplicated by the naff bitmap.
__global__ void k_mark_seed(SolveArgs a, const uint32_t* __restrict__ delu, const uint32_t* __restrict__ delv,
                            uint64_t nd, const uint32_t* __restrict__ insu, uint64_t ni) {
  State* st = a.st;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nd + ni;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t u = i < nd ? delu[i] : insu[i - nd];
    if (test_and_set(a.naff, u)) push(a.xl, &st->xcnt, u);
    if (i < nd) {
      const uint32_t v = delv[i];
      if (test_and_set(a.vaff, v)) {
        const int c = in_class(a.xtoff, v, a.mid_max);
        push(a.list[0][c], &st->cnt[0][c], v);
      }
    }
  }
}

// Mark the out-neighbours of each listed vertex, one warp per vertex.
//   SRC == EXPAND_XL            initial marking: xl -> lists[0]
//   SRC == EXPAND_XL_INTO_NEXT  inside the loop: xl -> lists[p^1]
//   SRC == EXPAND_FRONTIER      DT closure: fr[cur] -> lists[0] and fr[cur^1]
template <int SRC>
__global__ void __launch_bounds__(kThreads) k_expand(SolveArgs a, int cur) {
  State* st = a.st;
  if (SRC == EXPAND_XL_INTO_NEXT && st->done) return;
  const uint32_t* src;
  uint32_t count;
  int dst;
  if (SRC == EXPAND_FRONTIER) { src = a.fr[cur]; count = st->fcnt[cur]; dst = 0; }
  else { src = a.xl; count = st->xcnt; dst = SRC == EXPAND_XL ? 0 : ((st->iter & 1) ^ 1); }
  const uint32_t lane = lane_id();
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = warp; i < count; i += nwarps) {
    const uint32_t u = src[i];
    const uint32_t e = a.xoff[u + 1];
    for (uint32_t j = a.xoff[u] + lane; j < e; j += 32) {
      const uint32_t w = a.xedg[j];
      if (test_and_set(a.vaff, w)) {
        const int c = in_class(a.xtoff, w, a.mid_max);
        push(a.list[dst][c], &st->cnt[dst][c], w);
        if (SRC == EXPAND_FRONTIER) push(a.fr[cur ^ 1], &st->fcnt[cur ^ 1], w);
      }
    }
  }
}

// DT closure starts from every vertex of the DF marking (naff <- vaff,
// inc/pagerankCuda.hxx:442).
__global__ void k_frontier_from_lists(SolveArgs a) {
  State* st = a.st;
  const uint32_t n0 = st->cnt[0][0], n1 = st->cnt[0][1], n2 = st->cnt[0][2];
  const uint32_t total = n0 + n1 + n2;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    a.fr[0][i] = i < n0 ? a.list[0][0][i] : (i < n0 + n1 ? a.list[0][1][i - n0] : a.list[0][2][i - n0 - n1]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) st->fcnt[0] = total;
}

// After the update kernels of a dynamic iteration: make the new ranks current
// (the reference's swap, :688), refresh the contributions, keep the vertices
// still affected in the next lists and queue the ones to expand.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_commit(SolveArgs a) {
  constexpr bool FRONTIER = MODE >= PRX_DYNAMIC_FRONTIER;
  constexpr bool FIXED = MODE == PRX_DYNAMIC_TRAVERSAL;
  State* st = a.st;
  if (st->done) return;
  const int p = FIXED ? 0 : (st->iter & 1);
  const uint32_t n0 = st->cnt[p][0], n1 = st->cnt[p][1], n2 = st->cnt[p][2];
  const uint32_t total = n0 + n1 + n2;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int c = i < n0 ? 0 : (i < n0 + n1 ? 1 : 2);
    const uint32_t v = a.list[p][c][i - (c == 0 ? 0 : (c == 1 ? n0 : n0 + n1))];
    const double av = a.r[1][v];
    a.r[0][v] = av;
    a.c[0][v] = av / (double)a.xtdat[v];
    if (FRONTIER) {
      const uint8_t f = a.uflags[v];
      if (!(f & 1)) push(a.list[p ^ 1][c], &st->cnt[p ^ 1][c], v);
      if (f & 2) push(a.xl, &st->xcnt, v);
    }
  }
}

__global__ void k_flags_from_bitmap(const uint32_t* __restrict__ bm, uint8_t* __restrict__ out, uint32_t n) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    out[v] = (bm[v >> 5] >> (v & 31)) & 1u;
}

__global__ void k_state_reset(State* st, int max_iter, double tol) {
  st->el_bits[0] = st->el_bits[1] = 0;
  st->iter = 0;
  st->done = max_iter <= 0;  // while (l < L) runs no sweep when L <= 0
  st->max_iter = max_iter;
  st->tol = tol;
  st->last_delta = 0;
  for (int p = 0; p < 2; ++p)
    for (int c = 0; c < NCLS; ++c) st->cnt[p][c] = 0;
  st->xcnt = 0;
  st->fcnt[0] = st->fcnt[1] = 0;
  st->err = 0;
  st->edges = 0;
}

// ---- launchers ------------------------------------------------------------------
void launch_mark_seed(const SolveArgs& a, const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                      const uint32_t* insu, uint64_t ni, int sms, cudaStream_t s) {
  const uint64_t want = (nd + ni + kThreads - 1) / kThreads;
  const int grid = (int)(want < (uint64_t)sms * 8 ? (want ? want : 1) : (uint64_t)sms * 8);
  k_mark_seed<<<grid, kThreads, 0, s>>>(a, delu, delv, nd, insu, ni);
}

void launch_expand(const SolveArgs& a, int which, int sms, cudaStream_t s) {
  // `which` is an ExpandSrc; for EXPAND_FRONTIER the frontier parity is
  // passed in the high bits (which = EXPAND_FRONTIER | cur << 8).
  const int src = which & 0xff, cur = which >> 8;
  if (src == EXPAND_XL) k_expand<EXPAND_XL><<<sms * 4, kThreads, 0, s>>>(a, 0);
  else if (src == EXPAND_XL_INTO_NEXT) k_expand<EXPAND_XL_INTO_NEXT><<<sms * 4, kThreads, 0, s>>>(a, 0);
  else k_expand<EXPAND_FRONTIER><<<sms * 4, kThreads, 0, s>>>(a, cur);
}

void launch_frontier_from_lists(const SolveArgs& a, int sms, cudaStream_t s) {
  k_frontier_from_lists<<<sms * 4, kThreads, 0, s>>>(a);
}

void launch_commit(const SolveArgs& a, int mode, int sms, cudaStream_t s) {
  switch (mode) {
    case PRX_DYNAMIC_TRAVERSAL: k_commit<PRX_DYNAMIC_TRAVERSAL><<<sms * 8, kThreads, 0, s>>>(a); break;
    case PRX_DYNAMIC_FRONTIER: k_commit<PRX_DYNAMIC_FRONTIER><<<sms * 8, kThreads, 0, s>>>(a); break;
    default: k_commit<PRX_PRUNE_DYNAMIC_FRONTIER><<<sms * 8, kThreads, 0, s>>>(a); break;
  }
}

void launch_flags_from_bitmap(const uint32_t* bm, uint8_t* out, uint32_t n, cudaStream_t s) {
  const uint32_t grid = (n + kThreads - 1) / kThreads;
  k_flags_from_bitmap<<<grid < 4096 ? (grid ? grid : 1) : 4096, kThreads, 0, s>>>(bm, out, n);
}

void launch_state_reset(State* st, int max_iter, double tol, cudaStream_t s) {
  k_state_reset<<<1, 1, 0, s>>>(st, max_iter, tol);
}

}  // namespace prx
