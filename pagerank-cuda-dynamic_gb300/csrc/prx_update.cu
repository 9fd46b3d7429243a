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
#include "prx_device.cuh"

namespace prx {

template <int MODE> struct ModeTraits {
  static constexpr bool DYN = MODE >= PRX_DYNAMIC_TRAVERSAL;
  static constexpr bool FRONTIER = MODE >= PRX_DYNAMIC_FRONTIER;
  static constexpr bool PRUNE = MODE == PRX_PRUNE_DYNAMIC_FRONTIER;
  static constexpr bool FIXED_LISTS = MODE == PRX_DYNAMIC_TRAVERSAL;
};

// Finish vertex v given its contribution sum; returns |a_v - r_v| as bits.
template <int MODE>
__device__ __forceinline__ unsigned long long finish_vertex(const SolveArgs& a, uint32_t v, double cv, int p) {
  using T = ModeTraits<MODE>;
  const uint32_t d = a.xtdat[v];
  const double rv = T::DYN ? a.r[0][v] : a.r[p][v];
  double av;
  if (T::PRUNE) av = fma(a.P, cv - rv / (double)d, a.C0) * (1 / (1 - (a.P / (double)d)));
  else          av = fma(a.P, cv, a.C0);
  const double ev = fabs(av - rv);
  if (T::DYN) {
    a.r[1][v] = av;
    if (T::FRONTIER) {
      const double rel = ev / fmax(rv, av);
      uint8_t f = 0;
      if (T::PRUNE && rel <= a.C) { f |= 1; clear_bit(a.vaff, v); }
      if (rel > a.D) f |= 2;
      a.uflags[v] = f;
    }
  } else {
    a.r[p ^ 1][v] = av;
    a.c[p ^ 1][v] = av / (double)d;
  }
  return dbits(ev);
}

template <int MODE>
__device__ __forceinline__ void list_of(const SolveArgs& a, int cls, uint32_t begin, uint32_t count_static, int p,
                                        const uint32_t*& list, uint32_t& count) {
  using T = ModeTraits<MODE>;
  if (T::DYN) {
    const int q = T::FIXED_LISTS ? 0 : p;
    list = a.list[q][cls];
    count = a.st->cnt[q][cls];
  } else {
    list = a.cls_list + begin;
    count = count_static;
  }
}

// ---- LOW: thread per vertex -------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_update_low(SolveArgs a, uint32_t begin, uint32_t count_static) {
  using T = ModeTraits<MODE>;
  if (a.st->done) return;
  const int p = a.st->iter & 1;
  const uint32_t* list;
  uint32_t count;
  list_of<MODE>(a, LOW, begin, count_static, p, list, count);
  const double* __restrict__ c = T::DYN ? a.c[0] : a.c[p];
  const uint32_t* __restrict__ xtedg = a.xtedg;
  unsigned long long emax = 0, edges = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const uint32_t v = list[i];
    const uint32_t s = a.xtoff[v], e = a.xtoff[v + 1];
    double acc = 0.0;
    uint32_t j = s;
    for (; j + 4 <= e; j += 4) {
      const uint32_t u0 = __ldg(xtedg + j), u1 = __ldg(xtedg + j + 1);
      const uint32_t u2 = __ldg(xtedg + j + 2), u3 = __ldg(xtedg + j + 3);
      const double c0 = __ldg(c + u0), c1 = __ldg(c + u1), c2 = __ldg(c + u2), c3 = __ldg(c + u3);
      acc += c0; acc += c1; acc += c2; acc += c3;
    }
    for (; j < e; ++j) acc += __ldg(c + __ldg(xtedg + j));
    const unsigned long long ev = finish_vertex<MODE>(a, v, acc, p);
    emax = ev > emax ? ev : emax;
    edges += e - s;
  }
  block_max_bits(emax, &a.st->el_bits[p]);
  if (T::DYN) block_sum_u64(edges, &a.st->edges);
}

// ---- MID: warp per vertex, 256 virtual threads --------------------------------
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_update_mid(SolveArgs a, uint32_t begin, uint32_t count_static) {
  using T = ModeTraits<MODE>;
  if (a.st->done) return;
  const int p = a.st->iter & 1;
  const uint32_t* list;
  uint32_t count;
  list_of<MODE>(a, MID, begin, count_static, p, list, count);
  const double* __restrict__ c = T::DYN ? a.c[0] : a.c[p];
  const uint32_t lane = lane_id();
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long emax = 0, edges = 0;
  for (uint32_t i = warp; i < count; i += nwarps) {
    const uint32_t v = list[i];
    const uint32_t s = a.xtoff[v], d = a.xtoff[v + 1] - s;
    const uint32_t* __restrict__ ed = a.xtedg + s;
    double ps[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) ps[k] = 0.0;
    for (uint32_t base = 0; base < d; base += 256) {
      uint32_t u[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const uint32_t t = base + lane + 32u * k;
        u[k] = t < d ? __ldg(ed + t) : 0u;
      }
      double x[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = (base + lane + 32u * k < d) ? __ldg(c + u[k]) : 0.0;
#pragma unroll
      for (int k = 0; k < 8; ++k) ps[k] += x[k];
    }
    // halving tree over virtual thread t = lane + 32k
    ps[0] += ps[4]; ps[1] += ps[5]; ps[2] += ps[6]; ps[3] += ps[7];  // t < 128: += t+128
    ps[0] += ps[2]; ps[1] += ps[3];                                  // t < 64:  += t+64
    ps[0] += ps[1];                                                  // t < 32:  += t+32
    double x = ps[0];
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) {
      const unsigned long long ev = finish_vertex<MODE>(a, v, x, p);
      emax = ev > emax ? ev : emax;
      edges += d;
    }
  }
  block_max_bits(emax, &a.st->el_bits[p]);
  if (T::DYN) block_sum_u64(edges, &a.st->edges);
}

// ---- HIGH: block of 256 per vertex ------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(256) k_update_high(SolveArgs a, uint32_t begin, uint32_t count_static) {
  using T = ModeTraits<MODE>;
  __shared__ double part[256];
  if (a.st->done) return;
  const int p = a.st->iter & 1;
  const uint32_t* list;
  uint32_t count;
  list_of<MODE>(a, HIGH, begin, count_static, p, list, count);
  const double* __restrict__ c = T::DYN ? a.c[0] : a.c[p];
  const uint32_t t = threadIdx.x;
  unsigned long long emax = 0, edges = 0;
  for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
    const uint32_t v = list[i];
    const uint32_t s = a.xtoff[v], d = a.xtoff[v + 1] - s;
    const uint32_t* __restrict__ ed = a.xtedg + s;
    double acc = 0.0;
    uint32_t j = t;
    for (; j + 7 * 256 < d; j += 8 * 256) {
      uint32_t u[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) u[k] = __ldg(ed + j + 256 * k);
      double x[8];
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
      double x = part[t] + part[t + 32];
#pragma unroll
      for (int o = 16; o; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (t == 0) {
        const unsigned long long ev = finish_vertex<MODE>(a, v, x, p);
        emax = ev > emax ? ev : emax;
        edges += d;
      }
    }
    __syncthreads();
  }
  block_max_bits(emax, &a.st->el_bits[p]);
  if (T::DYN) block_sum_u64(edges, &a.st->edges);
}

// ---- init / finalize ----------------------------------------------------------
__global__ void k_init_ranks(SolveArgs a, const double* __restrict__ q) {
  // pagerankInitializeRanksCukW (inc/pagerankCuda.hxx:232-239) or the copy of
  // the previous ranks (:810,817), plus the contributions r/outdeg.
  const double r0 = 1.0 / (double)a.n;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
    const double r = q ? q[v] : r0;
    a.r[0][v] = r;
    a.c[0][v] = r / (double)a.xtdat[v];
  }
}

template <bool DYN, bool FIXED>
__global__ void k_finalize(State* st) {
  if (st->done) return;
  const int p = st->iter & 1;
  const double el = __longlong_as_double((long long)st->el_bits[p]);
  st->last_delta = el;
  st->iter += 1;
  if (el < st->tol || st->iter >= st->max_iter) st->done = 1;  // pagerankLoopCuU :680,689
  st->el_bits[p ^ 1] = 0;
  if (DYN && !FIXED) {
    st->cnt[p][0] = st->cnt[p][1] = st->cnt[p][2] = 0;
    st->xcnt = 0;
  }
}

// ---- launchers ------------------------------------------------------------------
static inline int cap_grid(uint64_t want, int cap) { return (int)(want < (uint64_t)cap ? (want ? want : 1) : cap); }

void launch_init_ranks(const SolveArgs& a, const double* q, bool, cudaStream_t s) {
  k_init_ranks<<<cap_grid((a.n + kThreads - 1) / kThreads, 152 * 16), kThreads, 0, s>>>(a, q);
}

template <int MODE>
static bool update_class_t(const SolveArgs& a, const GraphDev& g, int cls, int sms, cudaStream_t s) {
  if (ModeTraits<MODE>::DYN) {
    // list lengths live on the device: fixed grids that stride over them
    if (cls == LOW) k_update_low<MODE><<<sms * 8, kThreads, 0, s>>>(a, 0, 0);
    else if (cls == MID) k_update_mid<MODE><<<sms * 4, kThreads, 0, s>>>(a, 0, 0);
    else k_update_high<MODE><<<sms * 2, 256, 0, s>>>(a, 0, 0);
    return true;
  }
  const uint32_t b = g.cls_begin[cls], cnt = g.cls_begin[cls + 1] - b;
  if (!cnt) return false;
  if (cls == LOW) k_update_low<MODE><<<cap_grid((cnt + kThreads - 1) / kThreads, sms * 8), kThreads, 0, s>>>(a, b, cnt);
  else if (cls == MID) k_update_mid<MODE><<<cap_grid((cnt + 7) / 8, sms * 8), kThreads, 0, s>>>(a, b, cnt);
  else k_update_high<MODE><<<cap_grid(cnt, sms * 4), 256, 0, s>>>(a, b, cnt);
  return true;
}

bool launch_update_class(const SolveArgs& a, const GraphDev& g, int mode, int cls, int sms, cudaStream_t s) {
  switch (mode) {
    case PRX_STATIC:
    case PRX_NAIVE_DYNAMIC: return update_class_t<PRX_STATIC>(a, g, cls, sms, s);
    case PRX_DYNAMIC_TRAVERSAL: return update_class_t<PRX_DYNAMIC_TRAVERSAL>(a, g, cls, sms, s);
    case PRX_DYNAMIC_FRONTIER: return update_class_t<PRX_DYNAMIC_FRONTIER>(a, g, cls, sms, s);
    default: return update_class_t<PRX_PRUNE_DYNAMIC_FRONTIER>(a, g, cls, sms, s);
  }
}

void launch_finalize(const SolveArgs& a, int mode, cudaStream_t s) {
  // DT keeps its affected lists for the whole loop; DF / DF-P rebuild them.
  if (mode < PRX_DYNAMIC_TRAVERSAL) k_finalize<false, false><<<1, 1, 0, s>>>(a.st);
  else if (mode == PRX_DYNAMIC_TRAVERSAL) k_finalize<true, true><<<1, 1, 0, s>>>(a.st);
  else k_finalize<true, false><<<1, 1, 0, s>>>(a.st);
}

}  // namespace prx
