// prx_ppr.cu -- batched personalized PageRank: up to 64 teleport vectors per
// column block, solved together.  No counterpart in the reference (its
// solvers take the uniform teleport (1-P)/N only, inc/pagerankCuda.hxx:679).
//
// Vector k teleports uniformly to its seed set S_k:
//   r_k = (1-P) t_k + P * A^T D^-1 r_k,   t_k = (1/|S_k|) sum_{s in S_k} e_s,
// iterated by Jacobi sweeps from r_k = t_k until the L-inf change over all
// vertices and vectors of one sweep is below the tolerance (the reference's
// convergence test, :680,689, taken over the whole block).
//
// Layout: ranks are vertex-major, 64 values per vertex (one 512-byte FP64 or
// 256-byte FP32 row), so every in-edge is one coalesced row gather; lane l of
// a warp owns columns 2l and 2l+1.  Contributions are not stored: each
// gathered row is scaled by the source's reciprocal out-degree in the fma.
//
// Precision:
//  - PRX_FP64: FP64 rows, FP64 sums.
//  - PRX_FP32_REFINE: defect correction as for the static solver -- an FP64
//    residual sweep from the FP64 base x (rho = C + P A^T D^-1 x - x, its
//    L-inf the convergence test), then FP32 sweeps of the correction
//    e' = rho + P A^T D^-1 e (FP32 rows, half the bytes), then x += e.  The
//    FP32 sweeps of a round stop when their change is below the tolerance or
//    below 2^-18 of the correction's size (FP32 cannot resolve more), or at
//    the iteration cap.
//
// Rows of in-degree up to low_max (64 by default): one warp per vertex.
// Longer rows are cut into segments of `seg` in-edges (512 by default); a
// block sums a segment (warp w a contiguous eighth of it) into a partial
// row, and a warp per long vertex adds its segments' partials in order and
// finishes the vertex.  Every sum has a fixed order for given low_max / seg,
// so results are deterministic; prx_autotune_ppr picks both per graph.
//
// Loop: by default the whole iteration loop of a column block is one CUDA
// graph launch -- a conditional WHILE node over FP64 sweeps, and for the
// refinement a nested WHILE node over the FP32 correction sweeps of each
// round -- whose condition kernels read the device control block, so the
// host waits once per block; prx_options.loop = PRX_LOOP_HOST runs the same
// kernels from a host loop that reads the control block back between batches
// of sweeps.  Both run the same kernels in the same order (same results).
#include <algorithm>
#include <vector>
#include "prx_ctx.h"
#include "prx_device.cuh"

namespace prx {

constexpr int kCols = 64;         // vectors per column block
constexpr uint32_t kSeg = 512;    // default in-edges per segment of a long row
constexpr int kSegWarps = 8;      // warps per segment block

enum PprMode { PPR_J64 = 0, PPR_R64 = 1, PPR_S32 = 2 };

struct PprWs {
  int device = 0;
  uint32_t n = 0;                 // vertices the row buffers hold
  bool has32 = false;
  double* x[2] = {nullptr, nullptr};   // FP64 ranks, [n][64], ping-pong (refinement: base, sweep output)
  float* rho = nullptr;                // FP32 refinement: residual [n][64]
  float* e[2] = {nullptr, nullptr};    // FP32 corrections, ping-pong
  double* part = nullptr;              // partial rows of the segments [nseg][64]
  size_t part_cap = 0;                 // in segments
  uint32_t* seg = nullptr;             // [2][seg_cap]: vertex, first edge
  size_t seg_cap = 0;
  uint32_t* segstart = nullptr;        // first segment of each long vertex (+ total)
  size_t segstart_cap = 0;
  uint32_t* big = nullptr;             // vertices above a low_max other than 64, and their scan
  size_t big_cap = 0;
  uint32_t* toff = nullptr;            // teleport entries by vertex: offsets (n+1)
  uint32_t* tent = nullptr;            // entries: vertex, column (sorted)
  double* tmass = nullptr;             // entry mass 1/|S_k|
  size_t t_cap = 0, tm_cap = 0;
  double* out = nullptr;               // device staging of the host output
  size_t out_cap = 0;
};

void ppr_free(PprWs* w) {
  if (!w) return;
  cudaSetDevice(w->device);
  for (int i = 0; i < 2; ++i) {
    cudaFree(w->x[i]);
    cudaFree(w->e[i]);
  }
  cudaFree(w->rho);
  cudaFree(w->part);
  cudaFree(w->seg);
  cudaFree(w->segstart);
  cudaFree(w->big);
  cudaFree(w->toff);
  cudaFree(w->tent);
  cudaFree(w->tmass);
  cudaFree(w->out);
  delete w;
}

struct PprArgs {
  const uint32_t* xtoff;
  const uint32_t* xtedg;
  const unsigned long long* xtbase;  // row segments (see GraphDev); null: one segment
  uint32_t seg_shift;
  const double* rcp;
  const float* rcp32;
  const uint32_t* toff;
  const uint32_t* tcol;           // column of each teleport entry
  const double* tmass;
  double* x[2];
  float* rho;
  float* e[2];
  const uint32_t* big;            // vertices with in-degree > low_max
  uint32_t nbig;
  uint32_t low_max;               // rows up to this in-degree: one warp per vertex
  uint32_t seg;                   // in-edges per segment of a longer row (a multiple of kSegWarps)
  const uint32_t* segstart;       // [nbig + 1]
  const uint32_t* seg_v;
  const uint32_t* seg_e;
  uint32_t nseg;
  double* part;
  State* st;
  uint32_t n;
  double P, Q;                    // damping, 1 - damping
};

template <int MODE> struct PprType { using S = double; using V2 = double2; };
template <> struct PprType<PPR_S32> { using S = float; using V2 = float2; };

template <int MODE>
__device__ __forceinline__ bool ppr_skip(const State* st) {
  return st->done || (MODE == PPR_S32 && st->inner_done);
}

// Source rows of this sweep.
template <int MODE>
__device__ __forceinline__ const typename PprType<MODE>::V2* ppr_src(const PprArgs& a, const State* st) {
  using V2 = typename PprType<MODE>::V2;
  if (MODE == PPR_J64) return reinterpret_cast<const V2*>(a.x[st->iter & 1]);
  if (MODE == PPR_R64) return reinterpret_cast<const V2*>(a.x[0]);
  return reinterpret_cast<const V2*>(a.e[st->k32 & 1]);
}

// acc += row(u) / outdeg(u) over the in-edges [s, e) of edg (v's segment of
// the in-CSR; lane: its two columns).
template <int MODE>
__device__ __forceinline__ void ppr_gather(const PprArgs& a, const typename PprType<MODE>::V2* __restrict__ src,
                                           const uint32_t* __restrict__ edg, uint32_t s, uint32_t e,
                                           typename PprType<MODE>::V2& acc) {
  using S = typename PprType<MODE>::S;
  using V2 = typename PprType<MODE>::V2;
  const S* __restrict__ rc;
  if constexpr (MODE == PPR_S32) rc = a.rcp32;
  else rc = a.rcp;
  const uint32_t lane = lane_id();
  uint32_t j = s;
  for (; j + 4 <= e; j += 4) {
    const uint32_t u0 = __ldg(edg + j), u1 = __ldg(edg + j + 1), u2 = __ldg(edg + j + 2), u3 = __ldg(edg + j + 3);
    const V2 g0 = __ldg(src + (size_t)u0 * (kCols / 2) + lane), g1 = __ldg(src + (size_t)u1 * (kCols / 2) + lane);
    const V2 g2 = __ldg(src + (size_t)u2 * (kCols / 2) + lane), g3 = __ldg(src + (size_t)u3 * (kCols / 2) + lane);
    const S y0 = __ldg(rc + u0), y1 = __ldg(rc + u1), y2 = __ldg(rc + u2), y3 = __ldg(rc + u3);
    acc.x = fma(g0.x, y0, acc.x); acc.y = fma(g0.y, y0, acc.y);
    acc.x = fma(g1.x, y1, acc.x); acc.y = fma(g1.y, y1, acc.y);
    acc.x = fma(g2.x, y2, acc.x); acc.y = fma(g2.y, y2, acc.y);
    acc.x = fma(g3.x, y3, acc.x); acc.y = fma(g3.y, y3, acc.y);
  }
  for (; j < e; ++j) {
    const uint32_t u = __ldg(edg + j);
    const V2 g = __ldg(src + (size_t)u * (kCols / 2) + lane);
    const S y = __ldg(rc + u);
    acc.x = fma(g.x, y, acc.x);
    acc.y = fma(g.y, y, acc.y);
  }
}

// Finish vertex v from its gathered sum (lane: columns 2l, 2l+1); returns the
// lane's L-inf term (bits of a double, or of a float for PPR_S32) and, for
// PPR_S32, the size of the new correction in *emag.
template <int MODE>
__device__ __forceinline__ unsigned long long ppr_finish(const PprArgs& a, const State* st, uint32_t v,
                                                         typename PprType<MODE>::V2 acc, unsigned int* emag) {
  const uint32_t lane = lane_id();
  const size_t at = (size_t)v * (kCols / 2) + lane;
  if constexpr (MODE == PPR_S32) {
    const int q = st->k32 & 1;
    const float2 r = reinterpret_cast<const float2*>(a.rho)[at];
    const float2 old = reinterpret_cast<const float2*>(a.e[q])[at];
    const float P = (float)a.P;
    float2 en;
    en.x = fmaf(P, acc.x, r.x);
    en.y = fmaf(P, acc.y, r.y);
    reinterpret_cast<float2*>(a.e[q ^ 1])[at] = en;
    *emag = __float_as_uint(fmaxf(fabsf(en.x), fabsf(en.y)));
    return __float_as_uint(fmaxf(fabsf(en.x - old.x), fabsf(en.y - old.y)));
  } else {
    double tx = 0.0, ty = 0.0;
    for (uint32_t i = __ldg(a.toff + v), ie = __ldg(a.toff + v + 1); i < ie; ++i) {
      const uint32_t col = __ldg(a.tcol + i);
      if ((col >> 1) == lane) {
        if (col & 1u) ty += __ldg(a.tmass + i);
        else tx += __ldg(a.tmass + i);
      }
    }
    double2 an;
    an.x = fma(a.P, acc.x, a.Q * tx);
    an.y = fma(a.P, acc.y, a.Q * ty);
    const int p = MODE == PPR_J64 ? (st->iter & 1) : 0;
    const double2 old = reinterpret_cast<const double2*>(a.x[p])[at];
    reinterpret_cast<double2*>(a.x[p ^ 1])[at] = an;
    const double dx = an.x - old.x, dy = an.y - old.y;
    if (MODE == PPR_R64) {
      float2 r;
      r.x = (float)dx;
      r.y = (float)dy;
      reinterpret_cast<float2*>(a.rho)[at] = r;
      reinterpret_cast<float2*>(a.e[0])[at] = r;
    }
    return dbits(fmax(fabs(dx), fabs(dy)));
  }
}

template <int MODE>
__device__ __forceinline__ void ppr_reduce(State* st, unsigned long long dmax, unsigned int emag) {
  if constexpr (MODE == PPR_S32) {
    block_max_u32((unsigned int)dmax, &st->el32_bits[st->k32 & 1]);
    block_max_u32(emag, &st->e32max_bits[st->k32 & 1]);
  } else {
    block_max_bits(dmax, &st->el_bits[st->iter & 1]);
  }
}

// In-degree <= 64: one warp per vertex.
template <int MODE>
__global__ void __launch_bounds__(256) k_ppr_low(PprArgs a) {
  using V2 = typename PprType<MODE>::V2;
  State* st = a.st;
  if (ppr_skip<MODE>(st)) return;
  const V2* __restrict__ src = ppr_src<MODE>(a, st);
  unsigned long long dmax = 0;
  unsigned int emag = 0;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < a.n; v += warps) {
    const uint64_t iv = seg_index(v, a.seg_shift);
    const uint32_t s = __ldg(a.xtoff + iv), e = __ldg(a.xtoff + iv + 1);
    if (e - s > a.low_max) continue;
    V2 acc;
    acc.x = 0;
    acc.y = 0;
    ppr_gather<MODE>(a, src, seg_edges(a.xtedg, a.xtbase, a.seg_shift, v), s, e, acc);
    unsigned int em = 0;
    const unsigned long long d = ppr_finish<MODE>(a, st, v, acc, &em);
    dmax = d > dmax ? d : dmax;
    emag = em > emag ? em : emag;
  }
  ppr_reduce<MODE>(st, dmax, emag);
}

// Segments of the long rows: block per segment, warp w sums the w-th eighth;
// the partial row is the warps' sums added in warp order.
template <int MODE>
__global__ void __launch_bounds__(kSegWarps * 32) k_ppr_seg(PprArgs a) {
  using V2 = typename PprType<MODE>::V2;
  __shared__ V2 sh[kSegWarps][32];
  const State* st = a.st;
  if (ppr_skip<MODE>(st)) return;
  const V2* __restrict__ src = ppr_src<MODE>(a, st);
  const uint32_t w = threadIdx.x >> 5, lane = lane_id();
  V2* part = reinterpret_cast<V2*>(a.part);
  for (uint32_t g = blockIdx.x; g < a.nseg; g += gridDim.x) {
    const uint32_t v = a.seg_v[g], s0 = a.seg_e[g];
    const uint32_t end = min(s0 + a.seg, a.xtoff[seg_index(v, a.seg_shift) + 1]);
    const uint32_t per = a.seg / kSegWarps;
    const uint32_t s = min(s0 + w * per, end), e = min(s + per, end);
    V2 acc;
    acc.x = 0;
    acc.y = 0;
    ppr_gather<MODE>(a, src, seg_edges(a.xtedg, a.xtbase, a.seg_shift, v), s, e, acc);
    sh[w][lane] = acc;
    __syncthreads();
    if (w == 0) {
      V2 t = sh[0][lane];
#pragma unroll
      for (int k = 1; k < kSegWarps; ++k) {
        t.x += sh[k][lane].x;
        t.y += sh[k][lane].y;
      }
      part[(size_t)g * (kCols / 2) + lane] = t;
    }
    __syncthreads();
  }
}

// Long rows: warp per vertex adds its segments' partial rows in order.
template <int MODE>
__global__ void __launch_bounds__(256) k_ppr_combine(PprArgs a) {
  using V2 = typename PprType<MODE>::V2;
  State* st = a.st;
  if (ppr_skip<MODE>(st)) return;
  const V2* part = reinterpret_cast<const V2*>(a.part);
  const uint32_t lane = lane_id();
  unsigned long long dmax = 0;
  unsigned int emag = 0;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < a.nbig; i += warps) {
    const uint32_t v = a.big[i];
    V2 acc;
    acc.x = 0;
    acc.y = 0;
    for (uint32_t g = a.segstart[i]; g < a.segstart[i + 1]; ++g) {
      const V2 t = part[(size_t)g * (kCols / 2) + lane];
      acc.x += t.x;
      acc.y += t.y;
    }
    unsigned int em = 0;
    const unsigned long long d = ppr_finish<MODE>(a, st, v, acc, &em);
    dmax = d > dmax ? d : dmax;
    emag = em > emag ? em : emag;
  }
  ppr_reduce<MODE>(st, dmax, emag);
}

// ---- loop control ------------------------------------------------------------
__global__ void k_ppr_fin64(State* st) {  // Jacobi FP64 sweep
  if (st->done) return;
  const int p = st->iter & 1;
  const double el = __longlong_as_double((long long)st->el_bits[p]);
  st->last_delta = el;
  st->iter += 1;
  st->el_bits[p ^ 1] = 0;
  if (el < st->tol || st->iter >= st->max_iter) st->done = 1;
}

__global__ void k_ppr_fin_r64(State* st) {  // refinement: FP64 residual sweep
  if (st->done) return;
  const double el = __longlong_as_double((long long)st->el_bits[st->iter & 1]);
  st->last_delta = el;
  st->iter += 1;
  st->rounds += 1;
  st->el_bits[0] = st->el_bits[1] = 0;
  if (el < st->tol || st->iter >= st->max_iter) {
    st->done = 1;
    return;
  }
  st->k32 = 0;
  st->inner_done = 0;
  st->el32_bits[0] = st->el32_bits[1] = 0;
  st->e32max_bits[0] = st->e32max_bits[1] = 0;
  st->el32_prev[0] = st->el32_prev[1] = 0;
}

__global__ void k_ppr_fin32(State* st) {  // refinement: FP32 correction sweep
  if (st->done || st->inner_done) return;
  const int q = st->k32 & 1;
  const float dl = __uint_as_float(st->el32_bits[q]);
  const float em = __uint_as_float(st->e32max_bits[q]);
  st->iter += 1;
  st->k32 += 1;
  st->el32_bits[q ^ 1] = 0;
  st->e32max_bits[q ^ 1] = 0;
  const float prev = __uint_as_float(st->el32_prev[0]), prev2 = __uint_as_float(st->el32_prev[1]);
  st->el32_prev[1] = st->el32_prev[0];
  st->el32_prev[0] = __float_as_uint(dl);
  if (dl < (float)st->tol || dl < em * 0x1p-18f || st->iter >= st->max_iter ||
      fp32_round_done(dl, prev, prev2, st->tol))
    st->inner_done = 1;
}

// x_b += e (the correction of the last FP32 sweep); nothing once the solve
// is done (the graph loop reaches it after a converged FP64 sweep).
__global__ void k_ppr_commit(PprArgs a) {
  if (a.st->done) return;
  const float* __restrict__ e = a.e[a.st->k32 & 1];
  const size_t total = (size_t)a.n * kCols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    a.x[0][i] += (double)e[i];
}

// Conditions of the graph-launched loops.  Each counts its own bodies and
// stops after `cap` of them whatever the other kernels did, so the loops end
// even if a finalize kernel never ran.
__global__ void k_ppr_cond(cudaGraphConditionalHandle h, State* st, int cap, int refine) {
  const int rounds = ++st->graph_rounds;
  const bool more = !st->done && (!refine || st->iter < st->max_iter) && rounds < cap;
  cudaGraphSetConditional(h, more ? 1u : 0u);
}
__global__ void k_ppr_arm_inner(cudaGraphConditionalHandle h, State* st) {
  st->graph_inner = 0;
  cudaGraphSetConditional(h, (!st->done && !st->inner_done) ? 1u : 0u);
}
__global__ void k_ppr_cond_inner(cudaGraphConditionalHandle h, State* st, int cap) {
  const int rounds = ++st->graph_inner;
  cudaGraphSetConditional(h, (!st->done && !st->inner_done && rounds < cap) ? 1u : 0u);
}

// ---- setup ---------------------------------------------------------------------
// toff[v] = first teleport entry of v (entries sorted by vertex).
__global__ void k_ppr_toff(const uint32_t* __restrict__ ent_v, uint32_t nent, uint32_t n, uint32_t* __restrict__ toff) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = nent;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (ent_v[mid] < v) lo = mid + 1;
      else hi = mid;
    }
    toff[v] = lo;
  }
}

// x0 = t (rows zeroed before): each vertex adds its own entries.
__global__ void k_ppr_init(PprArgs a) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x)
    for (uint32_t i = a.toff[v]; i < a.toff[v + 1]; ++i) a.x[0][(size_t)v * kCols + a.tcol[i]] += a.tmass[i];
}

// Segment counts of the long vertices (ceil(indeg / seg)), then the segments.
__global__ void k_ppr_segcount(const uint32_t* __restrict__ xtoff, uint32_t shift, const uint32_t* __restrict__ big,
                               uint32_t nbig, uint32_t seg, uint32_t* __restrict__ cnt) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nbig; i += gridDim.x * blockDim.x)
    cnt[i] = (row_len(xtoff, shift, big[i]) + seg - 1) / seg;
}

// Vertices of in-degree above t: flags (n + 1 entries, the last 0) for the
// scan, then the ascending list.
__global__ void k_ppr_bigflags(const uint32_t* __restrict__ xtoff, uint32_t shift, uint32_t n, uint32_t t,
                               uint32_t* __restrict__ f) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x)
    f[v] = v < n && row_len(xtoff, shift, v) > t ? 1u : 0u;
}
__global__ void k_ppr_biglist(const uint32_t* __restrict__ xtoff, uint32_t shift, uint32_t n, uint32_t t,
                              const uint32_t* __restrict__ pos, uint32_t* __restrict__ big) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    if (row_len(xtoff, shift, v) > t) big[pos[v]] = v;
}

// seg_e: the segment's first in-edge, relative to v's row segment like the
// offsets.
__global__ void k_ppr_segfill(const uint32_t* __restrict__ xtoff, uint32_t shift, const uint32_t* __restrict__ big,
                              uint32_t nbig, uint32_t seg, const uint32_t* __restrict__ start,
                              uint32_t* __restrict__ seg_v, uint32_t* __restrict__ seg_e) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nbig; i += gridDim.x * blockDim.x) {
    const uint32_t v = big[i];
    const uint32_t s0 = xtoff[seg_index(v, shift)];
    for (uint32_t g = start[i], k = 0; g < start[i + 1]; ++g, ++k) {
      seg_v[g] = v;
      seg_e[g] = s0 + k * seg;
    }
  }
}

// out[v * nvec + c0 + k] = x[v][k] for k < w.
__global__ void k_ppr_out(const double* __restrict__ x, uint32_t n, uint32_t nvec, uint32_t c0, uint32_t w,
                          double* __restrict__ out) {
  const size_t total = (size_t)n * w;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t v = i / w, k = i % w;
    out[v * nvec + c0 + k] = x[v * kCols + k];
  }
}

static inline int grid_for(uint64_t work, int threads, int cap) {
  const uint64_t b = (work + threads - 1) / threads;
  return (int)(b < 1 ? 1 : (b < (uint64_t)cap ? b : cap));
}

template <int MODE>
static void ppr_sweep(const PprArgs& a, int sms, cudaStream_t s, uint64_t& launches) {
  k_ppr_low<MODE><<<grid_for((uint64_t)a.n * 32, 256, sms * 8), 256, 0, s>>>(a);
  ++launches;
  if (a.nseg) {
    k_ppr_seg<MODE><<<(int)std::min<uint64_t>(a.nseg, (uint64_t)sms * 8), kSegWarps * 32, 0, s>>>(a);
    k_ppr_combine<MODE><<<grid_for((uint64_t)a.nbig * 32, 256, sms * 8), 256, 0, s>>>(a);
    launches += 2;
  }
}

}  // namespace prx

// ---- host driver ---------------------------------------------------------------------
template <class T>
static cudaError_t grow(T** p, size_t& cap, size_t want) {
  if (*p && cap >= want) return cudaSuccess;
  cudaFree(*p);
  *p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(p, sizeof(T) * (want ? want : 1));
  if (e == cudaSuccess) cap = want;
  return e;
}

static int ppr_ws(prx_context* c, uint32_t n, bool fp32) {
  if (!c->ppr) {
    c->ppr = new PprWs();
    c->ppr->device = c->device;
  }
  PprWs& w = *c->ppr;
  if (w.n < n) {
    for (int i = 0; i < 2; ++i) {
      cudaFree(w.x[i]); w.x[i] = nullptr;
      cudaFree(w.e[i]); w.e[i] = nullptr;
    }
    cudaFree(w.rho); w.rho = nullptr;
    cudaFree(w.toff); w.toff = nullptr;
    w.n = 0;
    w.has32 = false;
    const size_t rows = (size_t)n * kCols;
    for (int i = 0; i < 2; ++i) TRY_CUDA_ST(cudaMalloc(&w.x[i], sizeof(double) * rows));
    TRY_CUDA_ST(cudaMalloc(&w.toff, sizeof(uint32_t) * ((size_t)n + 1)));
    w.n = n;
  }
  if (fp32 && !w.has32) {
    const size_t rows = (size_t)w.n * kCols;
    TRY_CUDA_ST(cudaMalloc(&w.rho, sizeof(float) * rows));
    for (int i = 0; i < 2; ++i) TRY_CUDA_ST(cudaMalloc(&w.e[i], sizeof(float) * rows));
    w.has32 = true;
  }
  return PRX_OK;
}

// The long rows of graph g (in-degree above a.low_max) and their segments of
// a.seg edges into the workspace; returns the counts.
static int ppr_segments(prx_context* c, const GraphDev& g, PprArgs& a) {
  PprWs& w = *c->ppr;
  cudaStream_t s = c->stream;
  uint32_t nbig = 0;
  if (a.low_max == kLowMax) {  // the graph's MID and HIGH classes
    nbig = g.cls_begin[NCLS] - g.cls_begin[MID];
    a.big = g.cls_list + g.cls_begin[MID];
  } else {
    TRY_CUDA_ST(grow(&w.big, w.big_cap, 2 * ((size_t)g.n + 1)));
    uint32_t* pos = w.big + g.n + 1;
    k_ppr_bigflags<<<grid_for((uint64_t)g.n + 1, 256, c->sms * 16), 256, 0, s>>>(g.xtoff, g.seg_shift, g.n, a.low_max, pos);
    TRY_CUDA_ST(exclusive_scan_u32(pos, g.n + 1, s));
    k_ppr_biglist<<<grid_for(g.n, 256, c->sms * 16), 256, 0, s>>>(g.xtoff, g.seg_shift, g.n, a.low_max, pos, w.big);
    TRY_CUDA_ST(cudaMemcpyAsync(&nbig, pos + g.n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    TRY_CUDA_ST(cudaStreamSynchronize(s));
    a.big = w.big;
  }
  a.nbig = nbig;
  a.nseg = 0;
  if (!nbig) return PRX_OK;
  TRY_CUDA_ST(grow(&w.segstart, w.segstart_cap, (size_t)nbig + 1));
  const int grid = grid_for(nbig, 256, c->sms * 4);
  k_ppr_segcount<<<grid, 256, 0, s>>>(g.xtoff, g.seg_shift, a.big, nbig, a.seg, w.segstart);
  TRY_CUDA_ST(exclusive_scan_u32(w.segstart, nbig + 1, s));
  uint32_t nseg = 0;
  TRY_CUDA_ST(cudaMemcpyAsync(&nseg, w.segstart + nbig, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  TRY_CUDA_ST(cudaStreamSynchronize(s));
  TRY_CUDA_ST(grow(&w.seg, w.seg_cap, 2 * (size_t)nseg));
  TRY_CUDA_ST(grow(&w.part, w.part_cap, (size_t)nseg * kCols));
  k_ppr_segfill<<<grid, 256, 0, s>>>(g.xtoff, g.seg_shift, a.big, nbig, a.seg, w.segstart, w.seg, w.seg + nseg);
  a.segstart = w.segstart;
  a.seg_v = w.seg;
  a.seg_e = w.seg + nseg;
  a.nseg = nseg;
  a.part = w.part;
  return PRX_OK;
}

// Teleport entries of columns [c0, c0 + cols) sorted by (vertex, column).
static int ppr_teleport(prx_context* c, uint32_t n, const uint32_t* seed_off, const uint32_t* seeds, uint32_t c0,
                        uint32_t cols, PprArgs& a) {
  PprWs& w = *c->ppr;
  cudaStream_t s = c->stream;
  struct Ent { uint32_t v, col; double m; };
  std::vector<Ent> ent;
  ent.reserve(seed_off[c0 + cols] - seed_off[c0]);
  for (uint32_t k = 0; k < cols; ++k) {
    const uint32_t b = seed_off[c0 + k], e = seed_off[c0 + k + 1];
    const double m = 1.0 / (double)(e - b);
    for (uint32_t i = b; i < e; ++i) ent.push_back({seeds[i], k, m});
  }
  std::sort(ent.begin(), ent.end(), [](const Ent& x, const Ent& y) { return x.v != y.v ? x.v < y.v : x.col < y.col; });
  const size_t ne = ent.size();
  std::vector<uint32_t> hv(ne), hc(ne);
  std::vector<double> hm(ne);
  for (size_t i = 0; i < ne; ++i) {
    hv[i] = ent[i].v;
    hc[i] = ent[i].col;
    hm[i] = ent[i].m;
  }
  TRY_CUDA_ST(grow(&w.tent, w.t_cap, 2 * ne));
  TRY_CUDA_ST(grow(&w.tmass, w.tm_cap, ne));
  TRY_CUDA_ST(cudaMemcpyAsync(w.tent, hv.data(), 4 * ne, cudaMemcpyHostToDevice, s));
  TRY_CUDA_ST(cudaMemcpyAsync(w.tent + ne, hc.data(), 4 * ne, cudaMemcpyHostToDevice, s));
  TRY_CUDA_ST(cudaMemcpyAsync(w.tmass, hm.data(), 8 * ne, cudaMemcpyHostToDevice, s));
  k_ppr_toff<<<grid_for((uint64_t)n + 1, 256, c->sms * 16), 256, 0, s>>>(w.tent, (uint32_t)ne, n, w.toff);
  // the host vectors must outlive the copies
  TRY_CUDA_ST(cudaStreamSynchronize(s));
  a.toff = w.toff;
  a.tcol = w.tent + ne;
  a.tmass = w.tmass;
  return PRX_OK;
}

// Reads the control block back (one sync).
static int ppr_check(prx_context* c) {
  TRY_CUDA_ST(cudaGetLastError());
  TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, c->stream));
  TRY_CUDA_ST(cudaStreamSynchronize(c->stream));
  return PRX_OK;
}

// The iteration loop of one column block as one CUDA graph launch (see the
// file comment); on return st_host[1] holds the control block.  Kernel
// launches inside the graph are counted into *body_launches from the
// control block (FP64 sweeps, FP32 sweeps).
static int ppr_block_graph(prx_context* c, PprArgs& a, const prx_options& o, bool fp32, uint64_t* body_launches) {
  cudaStream_t s = c->stream, s2 = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int st = PRX_OK;
  const int cap = (o.max_iterations < (1 << 30) ? o.max_iterations : (1 << 30)) + 2;
  uint64_t sweep_l = 0, sweep32_l = 0;
  cudaError_t e = cudaGraphCreate(&graph, 0);
  cudaGraphConditionalHandle ho{}, hi{};
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&ho, graph, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = ho;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &p);
  if (e == cudaSuccess && fp32) e = cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(s, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                          cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t ec = cudaSuccess;
    if (!fp32) {
      ppr_sweep<PPR_J64>(a, c->sms, s, sweep_l);
      k_ppr_fin64<<<1, 1, 0, s>>>(a.st);
      k_ppr_cond<<<1, 1, 0, s>>>(ho, a.st, cap, 0);
    } else {
      // the inner handle belongs to the outer body, the graph being captured
      cudaStreamCaptureStatus cs;
      cudaGraph_t body = nullptr;
      const cudaGraphNode_t* deps = nullptr;
      const cudaGraphEdgeData* edata = nullptr;
      size_t ndeps = 0;
      ec = cudaStreamGetCaptureInfo(s, &cs, nullptr, &body, nullptr, nullptr, nullptr);
      if (ec == cudaSuccess) ec = cudaGraphConditionalHandleCreate(&hi, body, 0, 0);
      if (ec == cudaSuccess) {
        ppr_sweep<PPR_R64>(a, c->sms, s, sweep_l);
        k_ppr_fin_r64<<<1, 1, 0, s>>>(a.st);
        k_ppr_arm_inner<<<1, 1, 0, s>>>(hi, a.st);
        ec = cudaStreamGetCaptureInfo(s, &cs, nullptr, &body, &deps, &edata, &ndeps);
      }
      cudaGraphNodeParams pi{};
      pi.type = cudaGraphNodeTypeConditional;
      pi.conditional.handle = hi;
      pi.conditional.type = cudaGraphCondTypeWhile;
      pi.conditional.size = 1;
      cudaGraphNode_t inode;
      if (ec == cudaSuccess) ec = cudaGraphAddNode(&inode, body, deps, edata, ndeps, &pi);
      if (ec == cudaSuccess) ec = cudaStreamUpdateCaptureDependencies(s, &inode, nullptr, 1,
                                                                      cudaStreamSetCaptureDependencies);
      // the FP32 sweeps of a round: the inner body, captured on a second stream
      if (ec == cudaSuccess) ec = cudaStreamBeginCaptureToGraph(s2, pi.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                                cudaStreamCaptureModeThreadLocal);
      if (ec == cudaSuccess) {
        ppr_sweep<PPR_S32>(a, c->sms, s2, sweep32_l);
        k_ppr_fin32<<<1, 1, 0, s2>>>(a.st);
        k_ppr_cond_inner<<<1, 1, 0, s2>>>(hi, a.st, cap);
        const cudaError_t el = cudaGetLastError();
        cudaGraph_t inner = nullptr;
        ec = cudaStreamEndCapture(s2, &inner);
        if (ec == cudaSuccess) ec = el;
      }
      if (ec == cudaSuccess) {
        k_ppr_commit<<<grid_for((size_t)a.n * kCols, 256, c->sms * 16), 256, 0, s>>>(a);
        k_ppr_cond<<<1, 1, 0, s>>>(ho, a.st, cap, 1);
      }
    }
    const cudaError_t el = cudaGetLastError();
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(s, &captured);  // always leave capture mode
    if (e == cudaSuccess) e = ec;
    if (e == cudaSuccess) e = el;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error(std::string("prx_solve_ppr_batched (graph loop): ") + cudaGetErrorString(e));
    st = e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (s2) cudaStreamDestroy(s2);
  if (!st) {
    const State& h = c->st_host[1];
    if (!fp32) {
      *body_launches = (uint64_t)h.iter * (sweep_l + 2);
    } else {
      const uint64_t n64 = (uint64_t)h.rounds, n32 = (uint64_t)(h.iter - h.rounds);
      *body_launches = n64 * (sweep_l + 5) + n32 * (sweep32_l + 2);
    }
  }
  return st;
}

// One column block; the answer's FP64 rows are left in *answer.
static int ppr_block(prx_context* c, const GraphDev& g, PprArgs& a, const prx_options& o, bool fp32,
                     const double** answer, prx_ppr_result* res) {
  cudaStream_t s = c->stream;
  uint64_t& L = c->launches;
  const size_t rows = (size_t)g.n * kCols;
  TRY_CUDA_ST(cudaMemsetAsync(a.x[0], 0, sizeof(double) * rows, s));
  k_ppr_init<<<grid_for(g.n, 256, c->sms * 16), 256, 0, s>>>(a);
  launch_state_reset(c->st, o.max_iterations, o.tolerance, s);
  L += 2;
  int st;
  if (o.loop != PRX_LOOP_HOST && o.max_iterations > 0) {
    uint64_t body = 0;
    if ((st = ppr_block_graph(c, a, o, fp32, &body))) return st;
    L += body;
    res->graph_launches += 1;
    const State& h = c->st_host[1];
    if (!fp32) {
      *answer = a.x[h.iter & 1];
      res->fp64_sweeps += h.iter;
    } else {
      *answer = h.done ? a.x[1] : a.x[0];  // a converged (or capped) FP64 sweep, else the committed base
      res->fp64_sweeps += h.rounds;
      res->fp32_sweeps += h.iter - h.rounds;
      res->refinements += h.rounds;
    }
    res->iterations = std::max(res->iterations, h.iter);
    res->last_delta = std::max(res->last_delta, h.last_delta);
    return PRX_OK;
  }
  if (!fp32) {
    if (o.max_iterations > 0) {
      for (int k = 1;; k = std::min(2 * k, 16)) {
        for (int i = 0; i < k; ++i) {
          ppr_sweep<PPR_J64>(a, c->sms, s, L);
          k_ppr_fin64<<<1, 1, 0, s>>>(c->st);
          ++L;
        }
        if ((st = ppr_check(c))) return st;
        if (c->st_host[1].done) break;
      }
    } else if ((st = ppr_check(c))) {
      return st;
    }
    const State& h = c->st_host[1];
    *answer = a.x[h.iter & 1];
    res->fp64_sweeps += h.iter;
    res->iterations = std::max(res->iterations, h.iter);
    res->last_delta = std::max(res->last_delta, h.last_delta);
    return PRX_OK;
  }
  int fp64 = 0;
  if (o.max_iterations <= 0) {
    if ((st = ppr_check(c))) return st;
    *answer = a.x[0];
    return PRX_OK;
  }
  for (;;) {
    ppr_sweep<PPR_R64>(a, c->sms, s, L);
    k_ppr_fin_r64<<<1, 1, 0, s>>>(c->st);
    ++L;
    ++fp64;
    if ((st = ppr_check(c))) return st;
    if (c->st_host[1].done) {
      *answer = a.x[1];
      break;
    }
    for (int k = 1;; k = std::min(2 * k, 16)) {
      for (int i = 0; i < k; ++i) {
        ppr_sweep<PPR_S32>(a, c->sms, s, L);
        k_ppr_fin32<<<1, 1, 0, s>>>(c->st);
        ++L;
      }
      if ((st = ppr_check(c))) return st;
      if (c->st_host[1].inner_done) break;
    }
    k_ppr_commit<<<grid_for(rows, 256, c->sms * 16), 256, 0, s>>>(a);
    ++L;
    if (c->st_host[1].iter >= o.max_iterations) {
      TRY_CUDA_ST(cudaStreamSynchronize(s));
      *answer = a.x[0];
      break;
    }
  }
  const State& h = c->st_host[1];
  res->fp64_sweeps += fp64;
  res->fp32_sweeps += h.iter - fp64;
  res->refinements += h.rounds;
  res->iterations = std::max(res->iterations, h.iter);
  res->last_delta = std::max(res->last_delta, h.last_delta);
  return PRX_OK;
}

static int ppr_common(prx_context* c, prx_graph* gr, uint32_t nvec, const uint32_t* seed_off, const uint32_t* seeds,
                      const prx_options* opt, double* ranks_out, prx_ppr_result* res, bool device_out) {
  if (!c || !gr || gr->ctx != c) FAIL(PRX_EINVAL, "prx_solve_ppr_batched: bad context or graph");
  if (nvec == 0 || !seed_off || !seeds) FAIL(PRX_EINVAL, "prx_solve_ppr_batched: no teleport vectors");
  prx_options o;
  if (opt) o = *opt;
  else prx_options_default(&o);
  if (o.precision != PRX_FP64 && o.precision != PRX_FP32_REFINE)
    FAIL(PRX_EINVAL, "prx_solve_ppr_batched: unknown precision");
  if (!(o.damping >= 0 && o.damping < 1)) FAIL(PRX_EINVAL, "prx_solve_ppr_batched: damping must be in [0, 1)");
  const GraphDev& g = gr->g;
  if (seed_off[0] != 0) FAIL(PRX_EINVAL, "prx_solve_ppr_batched: seed_off[0] must be 0");
  for (uint32_t k = 0; k < nvec; ++k)
    if (seed_off[k + 1] <= seed_off[k]) FAIL(PRX_EINVAL, "prx_solve_ppr_batched: every seed set must be non-empty");
  for (uint32_t i = 0; i < seed_off[nvec]; ++i)
    if (seeds[i] >= g.n) FAIL(PRX_EINVAL, "prx_solve_ppr_batched: seed id out of range");
  prx_ppr_result r{};
  if (g.n == 0) {
    if (res) *res = r;
    return PRX_OK;
  }
  if (!ranks_out) FAIL(PRX_EINVAL, "prx_solve_ppr_batched: ranks_out is NULL");
  TRY_CUDA_ST(cudaSetDevice(c->device));
  const bool fp32 = o.precision == PRX_FP32_REFINE;
  int st = ppr_ws(c, g.n, fp32);
  if (st) return st;
  PprWs& w = *c->ppr;
  cudaStream_t s = c->stream;
  PprArgs a{};
  a.xtoff = g.xtoff;
  a.xtedg = g.xtedg;
  a.xtbase = g.xtbase;
  a.seg_shift = g.seg_shift;
  a.rcp = g.rcp;
  a.rcp32 = g.rcp32;
  a.x[0] = w.x[0];
  a.x[1] = w.x[1];
  a.rho = w.rho;
  a.e[0] = w.e[0];
  a.e[1] = w.e[1];
  a.st = c->st;
  a.n = g.n;
  a.P = o.damping;
  a.Q = 1.0 - o.damping;
  a.low_max = g.ppr_low_max ? g.ppr_low_max : kLowMax;
  a.seg = g.ppr_seg ? g.ppr_seg : kSeg;
  r.low_max = a.low_max;
  r.seg_edges = a.seg;
  if ((st = ppr_segments(c, g, a))) return st;
  double* out = ranks_out;
  const size_t total = (size_t)g.n * nvec;
  if (!device_out) {
    TRY_CUDA_ST(grow(&w.out, w.out_cap, total));
    out = w.out;
  }
  const uint64_t l0 = c->launches;
  TRY_CUDA_ST(cudaEventRecord(c->ev[0], s));
  for (uint32_t c0 = 0; c0 < nvec; c0 += kCols) {
    const uint32_t cols = std::min<uint32_t>(kCols, nvec - c0);
    if ((st = ppr_teleport(c, g.n, seed_off, seeds, c0, cols, a))) return st;
    const double* answer = nullptr;
    if ((st = ppr_block(c, g, a, o, fp32, &answer, &r))) return st;
    k_ppr_out<<<grid_for((uint64_t)g.n * cols, 256, c->sms * 16), 256, 0, s>>>(answer, g.n, nvec, c0, cols, out);
    c->launches += 1;
  }
  TRY_CUDA_ST(cudaEventRecord(c->ev[1], s));
  if (!device_out) TRY_CUDA_ST(cudaMemcpyAsync(ranks_out, out, sizeof(double) * total, cudaMemcpyDeviceToHost, s));
  TRY_CUDA_ST(cudaStreamSynchronize(s));
  TRY_CUDA_ST(cudaGetLastError());
  float ms = 0;
  TRY_CUDA_ST(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  r.time_ms = ms;
  r.kernel_launches = c->launches - l0;
  if (res) *res = r;
  return PRX_OK;
}

extern "C" {

int prx_solve_ppr_batched(prx_context* c, prx_graph* gr, uint32_t nvec, const uint32_t* seed_off,
                          const uint32_t* seeds, const prx_options* o, double* ranks_out, prx_ppr_result* res) {
  return ppr_common(c, gr, nvec, seed_off, seeds, o, ranks_out, res, false);
}

int prx_solve_ppr_batched_device(prx_context* c, prx_graph* gr, uint32_t nvec, const uint32_t* seed_off,
                                 const uint32_t* seeds, const prx_options* o, double* ranks_out,
                                 prx_ppr_result* res) {
  return ppr_common(c, gr, nvec, seed_off, seeds, o, ranks_out, res, true);
}

// Times short FP32-refined solves (64 teleport vectors of one seed each, 1
// FP64 and 5 FP32 sweeps, best of two) over the warp-per-vertex bound
// (64, 256, 1024) and the segment width (256, 512, 1024, 2048 in-edges), and
// keeps the fastest pair on the graph for its later solves.
int prx_autotune_ppr(prx_context* c, prx_graph* gr, prx_ppr_tune_result* out) {
  if (!c || !gr || gr->ctx != c) FAIL(PRX_EINVAL, "prx_autotune_ppr: bad context or graph");
  GraphDev& g = gr->g;
  prx_ppr_tune_result best{};
  if (g.n == 0) {
    if (out) *out = best;
    return PRX_OK;
  }
  TRY_CUDA_ST(cudaSetDevice(c->device));
  const uint32_t nvec = kCols;
  std::vector<uint32_t> off(nvec + 1), seeds(nvec);
  for (uint32_t k = 0; k < nvec; ++k) {
    off[k] = k;
    seeds[k] = (uint32_t)((uint64_t)k * g.n / nvec);
  }
  off[nvec] = nvec;
  double* ranks = nullptr;
  TRY_CUDA_ST(cudaMalloc(&ranks, sizeof(double) * (size_t)g.n * nvec));
  prx_options o;
  prx_options_default(&o);
  o.precision = PRX_FP32_REFINE;
  o.tolerance = 0.0;
  o.max_iterations = 6;
  const uint32_t lows[] = {64, 256, 1024}, segs[] = {256, 512, 1024, 2048};
  const uint32_t keep_low = g.ppr_low_max, keep_seg = g.ppr_seg;
  float best_ms = 0;
  int trials = 0, st = PRX_OK;
  for (uint32_t lo : lows) {
    for (uint32_t sg : segs) {
      g.ppr_low_max = lo;
      g.ppr_seg = sg;
      float ms = 0;
      for (int rep = 0; rep < 2 && !st; ++rep) {
        prx_ppr_result r{};
        st = ppr_common(c, gr, nvec, off.data(), seeds.data(), &o, ranks, &r, true);
        if (!st && (rep == 0 || r.time_ms < ms)) ms = r.time_ms;
      }
      if (st) break;
      ++trials;
      if (!best.trials || ms < best_ms) {
        best_ms = ms;
        best.low_max = lo;
        best.seg_edges = sg;
        best.trials = 1;
      }
    }
    if (st) break;
  }
  cudaFree(ranks);
  if (st) {
    g.ppr_low_max = keep_low;
    g.ppr_seg = keep_seg;
    return st;
  }
  g.ppr_low_max = best.low_max;
  g.ppr_seg = best.seg_edges;
  best.ms_per_solve = best_ms;
  best.trials = trials;
  if (out) *out = best;
  return PRX_OK;
}

}  // extern "C"
