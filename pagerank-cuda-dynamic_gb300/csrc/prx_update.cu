// prx_update.cu -- the synchronous pull rank update (FP64 drop-in path).
//
// One Jacobi sweep computes, for every vertex v to update,
//     c_v = sum_{u in in(v)} r[u] / outdeg(u)
//     a_v = C0 + P*c_v                                  (Static, ND, DT, DF)
//     a_v = (C0 + P*(c_v - r_v/d_v)) * (1/(1 - P/d_v))  (DF-P: closed-form self-loop)
// as pagerankUpdateRanksThreadCukU / pagerankUpdateRanksBlockCukU do
// (inc/pagerankCuda.hxx:87-109, 162-188).  The term r[u]/outdeg(u) is
// computed once per source vertex (the contribution array c[]) instead of
// once per edge; the value is the same correctly rounded quotient.  Sums are
// formed in the reference's order, so the results are bit-identical to a
// serial restatement of it:
//   LOW  (in-degree <= 64): one thread, front to back.
//   MID  (64 < d <= mid_max): one warp emulates the reference's 256 threads --
//        lane l owns virtual threads l+32k (k = 0..7), adds terms t, t+256, ...
//        of each, then runs the halving tree of sumValuesBlockReduceCudU
//        (inc/_cuda.hxx:541-551): levels 128, 64, 32 in registers, 16..1 by
//        warp shuffles.
//   HIGH (d > mid_max): one 256-thread block, exactly the reference layout,
//        with 8 gathers in flight per thread and shuffles for the last levels.
// The L-inf delta is folded in with one atomicMax per block, so no separate
// reduction pass (liNormDeltaInplaceCuW, inc/_cuda.hxx:926-934) is needed.
// C0 + P*x is written as fma(): nvcc contracts the reference's expression
// into one DFMA.
//
// Vertex order.  The LOW kernel walks vertex ids in order, one warp per 32
// consecutive ids, so neighbouring rows and their local gathers stay close.
// The dynamic modes (DT, DF, DF-P) keep the affected set as bitmaps and the
// ranks / contributions as a ping-pong pair, like Static: iteration k reads
// parity p and writes parity p^1 for the vertices it updates.  A vertex that
// was updated in k-1 but is not updated in k has a stale copy in parity p^1
// and is copied across (the only copies needed -- the reference copies every
// unaffected vertex, :94-96).  Three bitmaps rotate: cur (k), nxt (k+1),
// prev (k-1); the LOW kernel clears prev after reading it, which makes it the
// empty nxt of iteration k+1.
#include <algorithm>
#include <type_traits>
#include "prx_device.cuh"

namespace prx {

template <int MODE> struct ModeTraits {
  static constexpr bool F32 = (MODE & MODE_F32) != 0;
  static constexpr int BASE = MODE & ~MODE_F32;
  static constexpr bool REFINE = BASE == MODE_REFINE64;
  static constexpr bool DYN = !REFINE && BASE >= PRX_DYNAMIC_TRAVERSAL;
  static constexpr bool FRONTIER = DYN && BASE >= PRX_DYNAMIC_FRONTIER;
  static constexpr bool PRUNE = BASE == PRX_PRUNE_DYNAMIC_FRONTIER;
  using V = typename std::conditional<F32, float, double>::type;  // rank / contribution type
  // resident blocks of 256 per SM the LOW kernel is compiled (register
  // budget) and launched for: the dynamic modes' bookkeeping needs more than
  // 32 registers a thread
  static constexpr int LOW_BLOCKS = (DYN || F32) ? 6 : 8;
};

// Rank, contribution and carried-sum arrays of a mode: FP64 r / c / acc64,
// or for the FP32 dynamic phase e / ce / acc32.
template <int MODE>
__device__ __forceinline__ typename ModeTraits<MODE>::V* ranks_of(const SolveArgs& a, int p) {
  if constexpr (ModeTraits<MODE>::F32) return a.e[p];
  else return a.r[p];
}
template <int MODE>
__device__ __forceinline__ typename ModeTraits<MODE>::V* contribs_of(const SolveArgs& a, int p) {
  if constexpr (ModeTraits<MODE>::F32) return a.ce[p];
  else return a.c[p];
}
template <int MODE>
__device__ __forceinline__ typename ModeTraits<MODE>::V* carried_of(const SolveArgs& a) {
  if constexpr (ModeTraits<MODE>::F32) return a.acc32;
  else return a.acc64;
}

// Data parity read by an iteration: the refinement's FP64 sweep always reads
// the base ranks (parity 0) and writes parity 1.
template <int MODE>
__device__ __forceinline__ int data_parity(const State* st) {
  return ModeTraits<MODE>::REFINE ? 0 : (st->iter & 1);
}

__device__ __forceinline__ void set_bit(uint32_t* bm, uint32_t w) {
  const uint32_t bit = 1u << (w & 31u);
  if (!(bm[w >> 5] & bit)) atomicOr(&bm[w >> 5], bit);
}

// Finish vertex v given its contribution sum.  Returns |a_v - r_v| as bits
// (of a double; an FP32 change converts exactly).  survive (dynamic): v stays
// affected next iteration; changed (DF / DF-P): its relative change exceeded
// the frontier tolerance, so its out-neighbours become affected (:106-107,
// expanded after the sweep as at :686-687).  FP32 phase: *mag is raised to
// |a_v| (bits of a float).
template <int MODE>
__device__ __forceinline__ unsigned long long finish_vertex(const SolveArgs& a, uint32_t v,
                                                            typename ModeTraits<MODE>::V cv, int p, bool& survive,
                                                            bool& changed, unsigned int& mag) {
  using T = ModeTraits<MODE>;
  const uint32_t d = a.xtdat[v];
  if constexpr (T::F32) {
    const float P = (float)a.P, C0 = (float)a.C0, df = (float)d;
    const float rv = a.e[p][v];
    float av;
    // ce[p][v] is rv / df, formed when rv was (the same division)
    if (T::PRUNE) av = fmaf(P, cv - a.ce[p][v], C0) * (1.f / (1.f - P / df));
    else          av = fmaf(P, cv, C0);
    const float ev = fabsf(av - rv);
    a.e[p ^ 1][v] = av;
    a.ce[p ^ 1][v] = av / df;
    mag = max(mag, __float_as_uint(fabsf(av)));
    survive = true;
    changed = false;
    if (T::FRONTIER) {  // relative change against the tolerances, without the division
      const float m = fmaxf(rv, av);
      if (T::PRUNE && ev <= (float)a.C * m) survive = false;
      changed = ev > (float)a.D * m;
    }
    return dbits((double)ev);
  } else {
    const double y = a.rcp[v];
    const double rv = a.r[p][v];
    double av;
    // c[p][v] is div_count(rv, d, y), formed when rv was; pf: 1 / (1 - P/d)
    if (T::PRUNE) av = fma(a.P, cv - a.c[p][v], a.C0) * a.pf[v];
    else          av = fma(a.P, cv, a.C0);
    const double ev = fabs(av - rv);
    a.r[p ^ 1][v] = av;
    if (T::REFINE) {
      // residual of the base ranks, the first FP32 correction and its contribution
      const float rho = (float)(av - rv);
      a.rho[v] = rho;
      a.e[0][v] = rho;
      a.ce[0][v] = __fdividef(rho, (float)d);
    } else {
      a.c[p ^ 1][v] = div_count(av, d, y);
    }
    survive = true;
    changed = false;
    if constexpr (T::FRONTIER) {  // rel = ev / max(rv, av) compared with C and D
      const RelChange rc = rel_change(av, rv);
      if (T::PRUNE && quot_le(rc, a.C)) survive = false;  // :106
      changed = quot_gt(rc, a.D);                          // :107
    }
    return dbits(ev);
  }
}

// ---- LOW: one warp per 32 consecutive vertex ids ------------------------------
// One launch per source chunk (PASS_ONLY when the row-major CSR is used
// whole).  Pass k adds the row's chunk-k segment to the partial sum carried in
// acc64 (sources ascending, so the chunks come in the row's own order); the
// first pass also does the dynamic modes' per-iteration bookkeeping, the last
// one finishes the vertex.
enum Pass { PASS_ONLY = 0, PASS_FIRST = 1, PASS_INNER = 2, PASS_LAST = 3 };

// hot: the layout encodes hot sources (the FP64 modes); their contributions
// are gathered from a.ch[p].
template <int MODE, int PASS>
__global__ void __launch_bounds__(kThreads, ModeTraits<MODE>::LOW_BLOCKS)
    k_update_low(SolveArgs a, uint32_t vb, uint32_t ve, const unsigned long long* __restrict__ base, uint32_t shift,
                 const uint32_t* __restrict__ off, const uint32_t* __restrict__ edg, bool hot) {
  using T = ModeTraits<MODE>;
  constexpr bool FIRST = PASS == PASS_ONLY || PASS == PASS_FIRST;
  constexpr bool LAST = PASS == PASS_ONLY || PASS == PASS_LAST;
  using V = typename T::V;
  State* st = a.st;
  if (st->done) return;
  const int iter = st->iter, p = data_parity<MODE>(st);
  const V* __restrict__ c = contribs_of<MODE>(a, p);
  const V* __restrict__ ch = nullptr;
  if constexpr (!T::F32) ch = a.ch[p];
  uint32_t *cur = nullptr, *nxt = nullptr, *prev = nullptr;
  if (T::DYN) {
    cur = a.bm[iter % 3];
    nxt = a.bm[(iter + 1) % 3];
    prev = a.bm[(iter + 2) % 3];
  }
  const uint32_t lane = lane_id();
  // rows [vb, ve) (vb a multiple of 32); off is indexed from row vb
  const uint32_t words = (uint32_t)(((uint64_t)ve + 31) >> 5);
  unsigned long long emax = 0, edges = 0;
  unsigned int mag = 0;
  for (uint32_t w = (vb >> 5) + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < words;
       w += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (w << 5) | lane;
    bool mine = v < ve;
    if (T::DYN) {
      const uint32_t cw = cur[w];
      if (FIRST) {
        const uint32_t pw = prev[w];
        if (((pw & ~cw) >> lane) & 1u) {  // updated last iteration, not this one: refresh parity p^1
          ranks_of<MODE>(a, p ^ 1)[v] = ranks_of<MODE>(a, p)[v];
          contribs_of<MODE>(a, p ^ 1)[v] = contribs_of<MODE>(a, p)[v];
        }
        if (lane == 0) {
          if (T::F32 && cw) atomicOr(&a.ever[w], cw);
          if (pw) prev[w] = 0;  // becomes the empty nxt of iteration k+1
          // nf[p^1] was filled and expanded by iteration k-1; clear it for k+1
          if (T::FRONTIER && a.nf[p ^ 1][w]) a.nf[p ^ 1][w] = 0;
        }
      }
      mine = mine && ((cw >> lane) & 1u);
      if (!__any_sync(0xffffffffu, mine)) continue;
    }
    const bool low = mine && ((a.low_bm[w] >> lane) & 1u);
    if (T::DYN && FIRST && mine && !low) {  // affected MID / HIGH vertex: its own kernel updates it
      const uint32_t d = row_len(a.xtoff, a.seg_shift, v);
      const int cls = d <= a.mid_max ? MID : HIGH;
      push(a.list[0][cls], &st->cnt[0][cls], v);
    }
    // One thread per row: a row's terms must be added front to back (the
    // reference's order), and a whole row per lane keeps the warp's FP64 adds
    // for different rows running side by side.
    const uint64_t iv = seg_index(v, shift) - vb;
    const uint32_t s = mine ? off[iv] : 0, e = mine ? off[iv + 1] : 0;
    mine = low && (FIRST || LAST || s < e);
    bool survive = false, changed = false;
    V acc = V(0);
    if constexpr (T::F32) {
      if (mine) acc = lane_row_sum(c, seg_edges(edg, base, shift, v), s, e, FIRST ? V(0) : carried_of<MODE>(a)[v]);
    } else {  // the whole warp sums together
      const V init = (mine && !FIRST) ? carried_of<MODE>(a)[v] : V(0);
      acc = warp_row_sums(c, seg_edges(edg, base, shift, v), s, mine ? e : s, init, ch, hot, a.int_adds);
    }
    if (mine) {
      edges += e - s;
      if (LAST) {
        const unsigned long long ev = finish_vertex<MODE>(a, v, acc, p, survive, changed, mag);
        emax = ev > emax ? ev : emax;
      } else {
        carried_of<MODE>(a)[v] = acc;
      }
    }
    if (LAST && T::DYN) {
      const unsigned keep = __ballot_sync(0xffffffffu, mine && survive);
      if (lane == 0 && keep) atomicOr(&nxt[w], keep);
    }
    if (LAST && T::FRONTIER) {
      const unsigned ch = __ballot_sync(0xffffffffu, mine && changed);
      if (lane == 0 && ch) {
        atomicOr(&a.nf[p][w], ch);
        atomicAdd(&st->nfcnt, (uint32_t)__popc(ch));
      }
    }
  }
  if (LAST) block_max_bits(emax, &st->el_bits[iter & 1]);
  if (LAST && T::F32) block_max_u32(mag, &st->e32max_bits[iter & 1]);
  if (T::DYN) block_sum_u64(edges, &st->edges);
}

// MID / HIGH lists: Static and ND use the graph's class lists; the dynamic
// modes use the affected MID / HIGH vertices the LOW kernel queued.
template <int MODE>
__device__ __forceinline__ void list_of(const SolveArgs& a, int cls, uint32_t begin, uint32_t count_static,
                                        const uint32_t*& list, uint32_t& count) {
  if (ModeTraits<MODE>::DYN) {
    list = a.list[0][cls];
    count = a.st->cnt[0][cls];
  } else {
    list = a.cls_list + begin;
    count = count_static;
  }
}

template <int MODE>
__device__ __forceinline__ void finish_listed(const SolveArgs& a, uint32_t v, typename ModeTraits<MODE>::V x, int p,
                                              unsigned long long& emax, unsigned int& mag) {
  bool survive, changed;
  const unsigned long long ev = finish_vertex<MODE>(a, v, x, p, survive, changed, mag);
  emax = ev > emax ? ev : emax;
  if (ModeTraits<MODE>::DYN && survive) atomicOr(&a.bm[(a.st->iter + 1) % 3][v >> 5], 1u << (v & 31u));
  if (ModeTraits<MODE>::FRONTIER && changed) {
    atomicOr(&a.nf[p][v >> 5], 1u << (v & 31u));
    atomicAdd(&a.st->nfcnt, 1u);
  }
}

// ---- MID: warp per vertex, 256 virtual threads --------------------------------
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_update_mid(SolveArgs a, uint32_t begin, uint32_t count_static) {
  using T = ModeTraits<MODE>;
  if (a.st->done) return;
  const int p = data_parity<MODE>(a.st);
  const uint32_t* list;
  uint32_t count;
  list_of<MODE>(a, MID, begin, count_static, list, count);
  using V = typename T::V;
  const V* __restrict__ c = contribs_of<MODE>(a, p);
  const uint32_t lane = lane_id();
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long emax = 0, edges = 0;
  unsigned int mag = 0;
  for (uint32_t i = warp; i < count; i += nwarps) {
    const uint32_t v = list[i];
    const uint64_t iv = seg_index(v, a.seg_shift);
    const uint32_t s = a.xtoff[iv], d = a.xtoff[iv + 1] - s;
    const uint32_t* __restrict__ ed = seg_edges(a.xtedg, a.xtbase, a.seg_shift, v) + s;
    V ps[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) ps[k] = V(0);
    for (uint32_t base = 0; base < d; base += 256) {
      uint32_t u[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const uint32_t t = base + lane + 32u * k;
        u[k] = t < d ? __ldg(ed + t) : 0u;
      }
      V x[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = (base + lane + 32u * k < d) ? __ldg(c + u[k]) : V(0);
#pragma unroll
      for (int k = 0; k < 8; ++k) ps[k] += x[k];
    }
    // halving tree over virtual thread t = lane + 32k
    ps[0] += ps[4]; ps[1] += ps[5]; ps[2] += ps[6]; ps[3] += ps[7];  // t < 128: += t+128
    ps[0] += ps[2]; ps[1] += ps[3];                                  // t < 64:  += t+64
    ps[0] += ps[1];                                                  // t < 32:  += t+32
    V x = ps[0];
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) {
      finish_listed<MODE>(a, v, x, p, emax, mag);
      edges += d;
    }
  }
  block_max_bits(emax, &a.st->el_bits[a.st->iter & 1]);
  if (T::F32) block_max_u32(mag, &a.st->e32max_bits[a.st->iter & 1]);
  if (T::DYN) block_sum_u64(edges, &a.st->edges);
}

// ---- HIGH: block of 256 per vertex ------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(256) k_update_high(SolveArgs a, uint32_t begin, uint32_t count_static) {
  using T = ModeTraits<MODE>;
  using V = typename T::V;
  __shared__ V part[256];
  if (a.st->done) return;
  const int p = data_parity<MODE>(a.st);
  const uint32_t* list;
  uint32_t count;
  list_of<MODE>(a, HIGH, begin, count_static, list, count);
  const V* __restrict__ c = contribs_of<MODE>(a, p);
  const uint32_t t = threadIdx.x;
  unsigned long long emax = 0, edges = 0;
  unsigned int mag = 0;
  for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
    const uint32_t v = list[i];
    const uint64_t iv = seg_index(v, a.seg_shift);
    const uint32_t s = a.xtoff[iv], d = a.xtoff[iv + 1] - s;
    const uint32_t* __restrict__ ed = seg_edges(a.xtedg, a.xtbase, a.seg_shift, v) + s;
    V acc = V(0);
    uint32_t j = t;
    for (; j + 7 * 256 < d; j += 8 * 256) {
      uint32_t u[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) u[k] = __ldg(ed + j + 256 * k);
      V x[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = __ldg(c + u[k]);
#pragma unroll
      for (int k = 0; k < 8; ++k) acc += x[k];
    }
    for (; j < d; j += 256) acc += __ldg(c + __ldg(ed + j));
    part[t] = acc;
    __syncthreads();
    if (t < 128) part[t] += part[t + 128];
    __syncthreads();
    if (t < 64) part[t] += part[t + 64];
    __syncthreads();
    if (t < 32) {
      V x = part[t] + part[t + 32];
#pragma unroll
      for (int o = 16; o; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (t == 0) {
        finish_listed<MODE>(a, v, x, p, emax, mag);
        edges += d;
      }
    }
    __syncthreads();
  }
  block_max_bits(emax, &a.st->el_bits[a.st->iter & 1]);
  if (T::F32) block_max_u32(mag, &a.st->e32max_bits[a.st->iter & 1]);
  if (T::DYN) block_sum_u64(edges, &a.st->edges);
}

// ---- DF / DF-P expansion after the sweep (:686-687) ---------------------------
// Nothing to expand once the iteration has converged: the loop ends here.
__device__ __forceinline__ bool expansion_needed(const State* st) {
  return !st->done && !(__longlong_as_double((long long)st->el_bits[st->iter & 1]) < st->tol);
}

// Push: every changed vertex marks its out-neighbours; out-degree <= 64 in
// the thread, larger ones are queued for k_expand_big.
__global__ void __launch_bounds__(kThreads) k_expand_push(SolveArgs a) {
  State* st = a.st;
  if (!expansion_needed(st) || st->nfcnt > a.pull_threshold) return;
  const int p = st->iter & 1;
  uint32_t* nxt = a.bm[(st->iter + 1) % 3];
  const uint32_t* nf = a.nf[p];
  const uint32_t words = (a.n + 31) >> 5;
  const uint32_t lane = lane_id();
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += (gridDim.x * blockDim.x) >> 5) {
    if (!((nf[w] >> lane) & 1u)) continue;
    const uint32_t u = (w << 5) | lane;
    const uint64_t iu = seg_index(u, a.seg_shift);
    const uint32_t b = a.xoff[iu], e = a.xoff[iu + 1];
    if (e - b > kLowMax) {
      push(a.xb, &st->xbcnt, u);
      continue;
    }
    const uint32_t* ed = seg_edges(a.xedg, a.xbase, a.seg_shift, u);
    for (uint32_t j = b; j < e; ++j) set_bit(nxt, ed[j]);
  }
}

// Pull: a vertex not yet marked becomes affected when any in-neighbour
// changed (the same set as the push; cheaper when most vertices changed).
__global__ void __launch_bounds__(kThreads) k_expand_pull(SolveArgs a) {
  State* st = a.st;
  if (!expansion_needed(st) || st->nfcnt <= a.pull_threshold) return;
  const int p = st->iter & 1;
  uint32_t* nxt = a.bm[(st->iter + 1) % 3];
  const uint32_t* nf = a.nf[p];
  const uint32_t words = (a.n + 31) >> 5;
  const uint32_t lane = lane_id();
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t word = nxt[w];
    const uint32_t v = (w << 5) | lane;
    bool hit = false;
    if (v < a.n && !((word >> lane) & 1u)) {
      const uint64_t iv = seg_index(v, a.seg_shift);
      const uint32_t e = a.xtoff[iv + 1];
      const uint32_t* ed = seg_edges(a.xtedg, a.xtbase, a.seg_shift, v);
      for (uint32_t j = a.xtoff[iv]; j < e && !hit; ++j) {
        const uint32_t u = ed[j];
        hit = (nf[u >> 5] >> (u & 31u)) & 1u;
      }
    }
    const unsigned add = __ballot_sync(0xffffffffu, hit);
    if (lane == 0 && add) nxt[w] = word | add;  // this warp is the only writer of word w here
  }
}

// Block-wide expansion of queued high out-degree vertices into bitmap `target`
// (initial marking) or, with target < 0, into the next iteration's bitmap.
__global__ void __launch_bounds__(256) k_expand_big(SolveArgs a, int target) {
  State* st = a.st;
  if (target < 0 && !expansion_needed(st)) return;
  uint32_t* bm = target < 0 ? a.bm[(st->iter + 1) % 3] : a.bm[target];
  const uint32_t count = st->xbcnt;
  for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
    const uint32_t u = a.xb[i];
    const uint64_t iu = seg_index(u, a.seg_shift);
    const uint32_t e = a.xoff[iu + 1];
    const uint32_t* ed = seg_edges(a.xedg, a.xbase, a.seg_shift, u);
    for (uint32_t j = a.xoff[iu] + threadIdx.x; j < e; j += blockDim.x) set_bit(bm, ed[j]);
  }
}

// ---- init / finalize ----------------------------------------------------------
__global__ void k_init_ranks(SolveArgs a, const double* __restrict__ q, int both) {
  // pagerankInitializeRanksCukW (inc/pagerankCuda.hxx:232-239) or the copy of
  // the previous ranks (:810,817), plus the contributions r/outdeg.  The
  // dynamic modes fill both parities (a vertex never updated reads either).
  const double r0 = 1.0 / (double)a.n;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
    const double r = q ? q[v] : r0;
    const double c = div_count(r, a.xtdat[v], a.rcp[v]);
    a.r[0][v] = r;
    a.c[0][v] = c;
    if (both) {
      a.r[1][v] = r;
      a.c[1][v] = c;
    }
  }
}

template <bool DYN, bool F32>
__global__ void k_finalize(State* st) {
  if (st->done) return;
  const int p = st->iter & 1;
  const double el = __longlong_as_double((long long)st->el_bits[p]);
  st->last_delta = el;
  st->iter += 1;
  bool stop = el < st->tol || st->iter >= st->max_iter;  // pagerankLoopCuU :680,689
  if (F32) {  // FP32 phase: also stop at what FP32 ranks can resolve, or on the predicted next change
    const float prev = __uint_as_float(st->el32_prev[0]), prev2 = __uint_as_float(st->el32_prev[1]);
    st->el32_prev[1] = st->el32_prev[0];
    st->el32_prev[0] = __float_as_uint((float)el);
    stop = stop || el < (double)__uint_as_float(st->e32max_bits[p]) * 0x1p-18 ||
           fp32_round_done((float)el, prev, prev2, st->tol);
    st->e32max_bits[p ^ 1] = 0;
  }
  if (stop) st->done = 1;
  st->el_bits[p ^ 1] = 0;
  if (DYN) {
    st->cnt[0][MID] = st->cnt[0][HIGH] = 0;
    st->xcnt = 0;
    st->nfcnt = 0;
    st->xbcnt = 0;
  }
}

// ---- launchers ------------------------------------------------------------------
static inline int cap_grid(uint64_t want, int cap) { return (int)(want < (uint64_t)cap ? (want ? want : 1) : cap); }

void launch_init_ranks(const SolveArgs& a, const double* q, bool dynamic, cudaStream_t s) {
  k_init_ranks<<<cap_grid((a.n + kThreads - 1) / kThreads, 152 * 16), kThreads, 0, s>>>(a, q, dynamic ? 1 : 0);
}

__global__ void k_init_ranks32(SolveArgs a, const double* __restrict__ q) {
  const float r0 = 1.0f / (float)a.n;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
    const float r = q ? (float)q[v] : r0;
    const float c = r / (float)a.xtdat[v];
    a.e[0][v] = a.e[1][v] = r;
    a.ce[0][v] = a.ce[1][v] = c;
  }
}

// The DF-P factor with the same operations as the reference's
// (1 / (1 - P/d)) inline in the update (:104), so its bits are the same.
// DF-P's factor depends on the out-degree alone: it is formed once per degree
// below kPfTable (with RN(1/d) divided as rcp is, so the same bits), and the
// vertices look it up; only larger degrees divide (an FP64 division is many
// FP64 instructions on this part).
__global__ void k_prune_table(SolveArgs a) {
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < kPfTable; d += gridDim.x * blockDim.x)
    a.pf_tab[d] = 1 / (1 - div_count(a.P, d, 1.0 / (double)d));
}

__global__ void k_prune_factor(SolveArgs a) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
    const uint32_t d = a.xtdat[v];
    a.pf[v] = d < kPfTable ? a.pf_tab[d] : 1 / (1 - div_count(a.P, d, a.rcp[v]));
  }
}

void launch_prune_factor(const SolveArgs& a, cudaStream_t s) {
  k_prune_table<<<kPfTable / kThreads, kThreads, 0, s>>>(a);
  k_prune_factor<<<cap_grid((a.n + kThreads - 1) / kThreads, 152 * 16), kThreads, 0, s>>>(a);
}

void launch_init_ranks32(const SolveArgs& a, const double* q, cudaStream_t s) {
  k_init_ranks32<<<cap_grid((a.n + kThreads - 1) / kThreads, 152 * 16), kThreads, 0, s>>>(a, q);
}

__global__ void k_commit_dyn32(SolveArgs a, int parity) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
    double x = a.r[0][v];
    if ((a.ever[v >> 5] >> (v & 31u)) & 1u) {
      x = (double)a.e[parity][v];
      a.r[0][v] = x;
    }
    a.c[0][v] = div_count(x, a.xtdat[v], a.rcp[v]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {  // reopen the loop for the FP64 refinement
    State* st = a.st;
    st->done = st->iter >= st->max_iter;
    st->el_bits[0] = st->el_bits[1] = 0;
    st->k32 = 0;
    st->inner_done = 0;
    st->el32_bits[0] = st->el32_bits[1] = 0;
    st->e32max_bits[0] = st->e32max_bits[1] = 0;
    st->el32_prev[0] = st->el32_prev[1] = 0;
    st->cnt[0][MID] = st->cnt[0][HIGH] = 0;
    st->nfcnt = 0;
    st->xbcnt = 0;
  }
}

// Dense copy of the hot sources' contributions: ch[p][h] = c[p][hot_list[h]].
// parity < 0: the parity the running iteration wrote (launched after its
// update kernels, before k_finalize; nothing once the solve is done).
__global__ void k_hot_copy(SolveArgs a, int parity) {
  int p = parity;
  if (p < 0) {
    if (a.st->done) return;
    p = (a.st->iter & 1) ^ 1;
  }
  const double* __restrict__ c = a.c[p];
  double* __restrict__ ch = a.ch[p];
  for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < a.hot_n; h += gridDim.x * blockDim.x)
    ch[h] = c[a.hot_list[h]];
}

bool launch_hot_copy(const SolveArgs& a, int parity, int sms, cudaStream_t s) {
  if (!a.hot_n) return false;
  k_hot_copy<<<cap_grid((a.hot_n + kThreads - 1) / kThreads, sms * 8), kThreads, 0, s>>>(a, parity);
  return true;
}

void launch_commit_dyn32(const SolveArgs& a, int parity, cudaStream_t s) {
  k_commit_dyn32<<<cap_grid((a.n + kThreads - 1) / kThreads, 152 * 16), kThreads, 0, s>>>(a, parity);
}

template <int MODE>
static bool update_class_t(const SolveArgs& a, const GraphDev& g, int cls, const ChunkLayout* lay, int sms,
                           cudaStream_t s) {
  constexpr bool DYN = ModeTraits<MODE>::DYN;
  if (cls == LOW) {
    // static: skip when the graph has no LOW vertex; dynamic: always (the
    // first pass also maintains the bitmaps)
    if (!DYN && g.cls_begin[1] == g.cls_begin[0]) return false;
    if (!lay || (lay->K <= 1 && !lay->hot)) {
      const uint64_t words = ((uint64_t)g.n + 31) / 32;
      const int grid = cap_grid((words + 7) / 8, sms * ModeTraits<MODE>::LOW_BLOCKS);
      k_update_low<MODE, PASS_ONLY>
          <<<grid, kThreads, 0, s>>>(a, 0, g.n, g.xtbase, g.seg_shift, g.xtoff, g.xtedg, false);
      return true;
    }
    const bool hot = lay->hot && a.hot_n > 0;
    // one pass per source chunk (per row segment and chunk on segmented rows)
    const size_t nseg = lay->seg_off.empty() ? 1 : lay->seg_off.size();
    for (size_t q = 0; q < nseg; ++q) {
      const uint32_t v0 = nseg == 1 ? 0 : (uint32_t)(q << g.seg_shift);
      const uint32_t v1 = nseg == 1 ? g.n : (uint32_t)std::min<uint64_t>(g.n, ((uint64_t)q + 1) << g.seg_shift);
      const uint32_t* offs = nseg == 1 ? lay->off : lay->seg_off[q];
      const uint32_t* edg = nseg == 1 ? lay->edg : lay->seg_edg[q];
      const size_t row = (size_t)(v1 - v0) + 1;
      const int grid = cap_grid(((uint64_t)(v1 - v0) + 31) / 32 / 8 + 1, sms * ModeTraits<MODE>::LOW_BLOCKS);
      for (int k = 0; k < lay->K; ++k) {
        const uint32_t* off = offs + k * row;
        if (lay->K == 1)
          k_update_low<MODE, PASS_ONLY><<<grid, kThreads, 0, s>>>(a, v0, v1, nullptr, 32, off, edg, hot);
        else if (k == 0)
          k_update_low<MODE, PASS_FIRST><<<grid, kThreads, 0, s>>>(a, v0, v1, nullptr, 32, off, edg, hot);
        else if (k == lay->K - 1)
          k_update_low<MODE, PASS_LAST><<<grid, kThreads, 0, s>>>(a, v0, v1, nullptr, 32, off, edg, hot);
        else
          k_update_low<MODE, PASS_INNER><<<grid, kThreads, 0, s>>>(a, v0, v1, nullptr, 32, off, edg, hot);
      }
    }
    return true;
  }
  if (DYN) {
    if (cls == MID) k_update_mid<MODE><<<sms * 4, kThreads, 0, s>>>(a, 0, 0);
    else k_update_high<MODE><<<sms * 2, 256, 0, s>>>(a, 0, 0);
    return true;
  }
  const uint32_t b = g.cls_begin[cls], cnt = g.cls_begin[cls + 1] - b;
  if (!cnt) return false;
  if (cls == MID) k_update_mid<MODE><<<cap_grid((cnt + 7) / 8, sms * 8), kThreads, 0, s>>>(a, b, cnt);
  else k_update_high<MODE><<<cap_grid(cnt, sms * 4), 256, 0, s>>>(a, b, cnt);
  return true;
}

bool launch_update_class(const SolveArgs& a, const GraphDev& g, int mode, int cls, const ChunkLayout* lay, int sms,
                         cudaStream_t s) {
  switch (mode) {
    case PRX_STATIC:
    case PRX_NAIVE_DYNAMIC: return update_class_t<PRX_STATIC>(a, g, cls, lay, sms, s);
    case PRX_DYNAMIC_TRAVERSAL: return update_class_t<PRX_DYNAMIC_TRAVERSAL>(a, g, cls, lay, sms, s);
    case PRX_DYNAMIC_FRONTIER: return update_class_t<PRX_DYNAMIC_FRONTIER>(a, g, cls, lay, sms, s);
    case PRX_PRUNE_DYNAMIC_FRONTIER: return update_class_t<PRX_PRUNE_DYNAMIC_FRONTIER>(a, g, cls, lay, sms, s);
    case PRX_DYNAMIC_TRAVERSAL | MODE_F32:
      return update_class_t<PRX_DYNAMIC_TRAVERSAL | MODE_F32>(a, g, cls, lay, sms, s);
    case PRX_DYNAMIC_FRONTIER | MODE_F32:
      return update_class_t<PRX_DYNAMIC_FRONTIER | MODE_F32>(a, g, cls, lay, sms, s);
    default: return update_class_t<PRX_PRUNE_DYNAMIC_FRONTIER | MODE_F32>(a, g, cls, lay, sms, s);
  }
}

bool launch_refine_sweep64(const SolveArgs& a, const GraphDev& g, int cls, const ChunkLayout* lay, int sms,
                           cudaStream_t s) {
  return update_class_t<MODE_REFINE64>(a, g, cls, lay, sms, s);
}

void launch_expand_iteration(const SolveArgs& a, int sms, cudaStream_t s) {
  const uint64_t words = ((uint64_t)a.n + 31) / 32;
  const int grid = cap_grid((words + 7) / 8, sms * 8);
  k_expand_push<<<grid, kThreads, 0, s>>>(a);
  k_expand_pull<<<grid, kThreads, 0, s>>>(a);
  k_expand_big<<<sms * 4, 256, 0, s>>>(a, -1);
}

void launch_expand_big(const SolveArgs& a, int target, int sms, cudaStream_t s) {
  k_expand_big<<<sms * 4, 256, 0, s>>>(a, target);
}

void launch_finalize(const SolveArgs& a, int mode, cudaStream_t s) {
  if (mode & MODE_F32) k_finalize<true, true><<<1, 1, 0, s>>>(a.st);
  else if (mode < PRX_DYNAMIC_TRAVERSAL) k_finalize<false, false><<<1, 1, 0, s>>>(a.st);
  else k_finalize<true, false><<<1, 1, 0, s>>>(a.st);
}

}  // namespace prx
