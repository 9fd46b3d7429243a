// prx_refine.cu -- FP32 storage with FP64 refinement (Static, ND).
//
// Defect correction around the reference's Jacobi iteration
// (pagerankLoopCuU, inc/pagerankCuda.hxx:675-692):
//   0. FP32 sweeps of the ranks themselves from the initial ranks (a round
//      with x_b = 0, rho = C0 and e_0 = the initial ranks), committed as the
//      first base x_b; no FP64 sweep is spent on the far-from-converged start.
//   1. FP64 sweep from the base ranks x_b (the reference's update, its order
//      and fma; update kernels in MODE_REFINE64): a = C0 + P*A*(x_b/d), and
//      rho = a - x_b.  Its L-inf is the reference's convergence test; when
//      it is below tol, a is the answer.
//   2. FP32 sweeps of the correction: e_1 = rho, e_{k+1} = rho + P*A*(e_k/d).
//      x_b + e_k is the k-th Jacobi iterate from x_b, so the FP32 loop stops on
//      the same criterion, |e_{k+1} - e_k|_inf < tol, or once the change is
//      below 2^-18 of |e|_inf (row sums of up to 64 FP32 terms cannot resolve
//      more; the next FP64 residual takes over).  Contributions e/d are
//      stored and gathered in FP32 (4 bytes per edge instead of 8) and
//      accumulated in FP32.
//   3. x_b += e in FP64, back to 1.
// Every FP64 and FP32 sweep counts as one iteration against max_iterations.
#include <algorithm>
#include "prx_device.cuh"

namespace prx {

__device__ __forceinline__ unsigned int fbits(float x) { return __float_as_uint(x); }

// New correction of v; returns |change| and raises *mag to |e| (bits).
__device__ __forceinline__ unsigned int finish32(const SolveArgs& a, uint32_t v, float sum, int q, unsigned int* mag) {
  const float en = fmaf((float)a.P, sum, a.rho[v]);
  const float dl = fabsf(en - a.e[q][v]);
  a.e[q ^ 1][v] = en;
  a.ce[q ^ 1][v] = __fdividef(en, (float)a.xtdat[v]);
  *mag = max(*mag, fbits(fabsf(en)));
  return fbits(dl);
}

// The L-inf change and correction size of a sweep (every thread calls it).
__device__ __forceinline__ void reduce32(State* st, unsigned int dl, unsigned int mag) {
  const int q = st->k32 & 1;
  block_max_u32(dl, &st->el32_bits[q]);
  block_max_u32(mag, &st->e32max_bits[q]);
}

// LOW: one warp per 32 consecutive ids, one lane per vertex, one launch per
// source chunk (partial sums carried in acc32), as the FP64 kernel.
template <bool FIRST, bool LAST>
__global__ void __launch_bounds__(kThreads) k32_low(SolveArgs a, uint32_t vb, uint32_t ve,
                                                    const unsigned long long* __restrict__ base,
                                                    uint32_t shift, const uint32_t* __restrict__ off,
                                                    const uint32_t* __restrict__ edg) {
  State* st = a.st;
  if (st->done || st->inner_done) return;
  const int q = st->k32 & 1;
  const float* __restrict__ ce = a.ce[q];
  // rows [vb, ve) (vb a multiple of 32); off is indexed from row vb
  const uint32_t words = (uint32_t)(((uint64_t)ve + 31) >> 5);
  unsigned int emax = 0, mag = 0;
  for (uint32_t w = (vb >> 5) + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < words;
       w += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (w << 5) | lane_id();
    if (v >= ve || !((a.low_bm[w] >> lane_id()) & 1u)) continue;
    const uint64_t iv = seg_index(v, shift) - vb;
    const uint32_t s = off[iv], e = off[iv + 1];
    if (!FIRST && !LAST && s == e) continue;
    const float acc = lane_row_sum(ce, seg_edges(edg, base, shift, v), s, e, FIRST ? 0.f : a.acc32[v]);
    if (LAST) emax = max(emax, finish32(a, v, acc, q, &mag));
    else a.acc32[v] = acc;
  }
  if (LAST) reduce32(st, emax, mag);
}

// MID: warp per vertex, lane-strided sums folded by shuffles.
__global__ void __launch_bounds__(kThreads) k32_mid(SolveArgs a, uint32_t begin, uint32_t count) {
  State* st = a.st;
  if (st->done || st->inner_done) return;
  const int q = st->k32 & 1;
  const float* __restrict__ ce = a.ce[q];
  const uint32_t lane = lane_id();
  unsigned int emax = 0, mag = 0;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < count; i += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = a.cls_list[begin + i];
    const uint64_t iv = seg_index(v, a.seg_shift);
    const uint32_t s = a.xtoff[iv], d = a.xtoff[iv + 1] - s;
    const uint32_t* __restrict__ ed = seg_edges(a.xtedg, a.xtbase, a.seg_shift, v) + s;
    float acc = 0.f;
    for (uint32_t t = lane; t < d; t += 32) acc += __ldg(ce + __ldg(ed + t));
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) emax = max(emax, finish32(a, v, acc, q, &mag));
  }
  reduce32(st, emax, mag);
}

// HIGH: block per vertex.
__global__ void __launch_bounds__(256) k32_high(SolveArgs a, uint32_t begin, uint32_t count) {
  __shared__ float part[8];
  State* st = a.st;
  if (st->done || st->inner_done) return;
  const int q = st->k32 & 1;
  const float* __restrict__ ce = a.ce[q];
  unsigned int emax = 0, mag = 0;
  for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
    const uint32_t v = a.cls_list[begin + i];
    const uint64_t iv = seg_index(v, a.seg_shift);
    const uint32_t s = a.xtoff[iv], d = a.xtoff[iv + 1] - s;
    const uint32_t* __restrict__ ed = seg_edges(a.xtedg, a.xtbase, a.seg_shift, v) + s;
    float acc = 0.f;
    for (uint32_t t = threadIdx.x; t < d; t += 256) acc += __ldg(ce + __ldg(ed + t));
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane_id() == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
      float x = threadIdx.x < 8 ? part[threadIdx.x] : 0.f;
#pragma unroll
      for (int o = 4; o; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (threadIdx.x == 0) emax = max(emax, finish32(a, v, x, q, &mag));
    }
    __syncthreads();
  }
  reduce32(st, emax, mag);
}

// After the FP64 sweep: its L-inf decides (:689); otherwise start a round of
// FP32 sweeps.
__global__ void k_refine_finalize64(State* st) {
  if (st->done) return;
  const int p = st->iter & 1;
  const double el = __longlong_as_double((long long)st->el_bits[p]);
  st->last_delta = el;
  st->iter += 1;
  st->rounds += 1;
  st->el_bits[p ^ 1] = 0;
  st->el_bits[p] = 0;
  if (el < st->tol || st->iter >= st->max_iter) {
    st->done = 1;  // the answer is the FP64 sweep's output
    return;
  }
  st->k32 = 0;
  st->inner_done = 0;
  st->el32_bits[0] = st->el32_bits[1] = 0;
  st->e32max_bits[0] = st->e32max_bits[1] = 0;
  st->el32_prev[0] = st->el32_prev[1] = 0;
}

__global__ void k_finalize32(State* st) {
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

// Round 0: x_b = 0, rho = C0, e_0 = the initial ranks (FP32), ce_0 = e_0 / d.
__global__ void k_refine_round0(SolveArgs a) {
  const float c0 = (float)a.C0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
    const float x = (float)a.r[0][v];
    a.r[0][v] = 0.0;
    a.rho[v] = c0;
    a.e[0][v] = x;
    a.ce[0][v] = __fdividef(x, (float)a.xtdat[v]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    State* st = a.st;
    st->k32 = 0;
    st->inner_done = st->done;
    st->el32_bits[0] = st->el32_bits[1] = 0;
    st->e32max_bits[0] = st->e32max_bits[1] = 0;
    st->el32_prev[0] = st->el32_prev[1] = 0;
  }
}

// x_b += e (FP64), c_b = x_b / outdeg.  Nothing once the solve is done (the
// graph-launched loop reaches it after the FP64 sweep that converged).
__global__ void k_refine_commit(SolveArgs a) {
  if (a.st->done) return;
  const float* __restrict__ e = a.e[a.st->k32 & 1];
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
    const double x = a.r[0][v] + (double)e[v];
    a.r[0][v] = x;
    a.c[0][v] = div_count(x, a.xtdat[v], a.rcp[v]);
  }
}

static inline int cap_grid32(uint64_t want, int cap) { return (int)(want < (uint64_t)cap ? (want ? want : 1) : cap); }

bool launch_sweep32(const SolveArgs& a, const GraphDev& g, int cls, const ChunkLayout* lay, int sms, cudaStream_t s) {
  const uint32_t b = g.cls_begin[cls], cnt = g.cls_begin[cls + 1] - b;
  if (!cnt) return false;
  if (cls == LOW) {
    if (!lay || lay->K <= 1) {
      const uint64_t words = ((uint64_t)g.n + 31) / 32;
      const int grid = cap_grid32((words + 7) / 8, sms * 8);
      k32_low<true, true><<<grid, kThreads, 0, s>>>(a, 0, g.n, g.xtbase, g.seg_shift, g.xtoff, g.xtedg);
      return true;
    }
    // one pass per source chunk (per row segment and chunk on segmented rows)
    const size_t nseg = lay->seg_off.empty() ? 1 : lay->seg_off.size();
    for (size_t q = 0; q < nseg; ++q) {
      const uint32_t v0 = nseg == 1 ? 0 : (uint32_t)(q << g.seg_shift);
      const uint32_t v1 = nseg == 1 ? g.n : (uint32_t)std::min<uint64_t>(g.n, ((uint64_t)q + 1) << g.seg_shift);
      const uint32_t* offs = nseg == 1 ? lay->off : lay->seg_off[q];
      const uint32_t* edg = nseg == 1 ? lay->edg : lay->seg_edg[q];
      const size_t row = (size_t)(v1 - v0) + 1;
      const int grid = cap_grid32(((uint64_t)(v1 - v0) + 31) / 32 / 8 + 1, sms * 8);
      for (int k = 0; k < lay->K; ++k) {
        const uint32_t* off = offs + k * row;
        if (k == 0) k32_low<true, false><<<grid, kThreads, 0, s>>>(a, v0, v1, nullptr, 32, off, edg);
        else if (k == lay->K - 1) k32_low<false, true><<<grid, kThreads, 0, s>>>(a, v0, v1, nullptr, 32, off, edg);
        else k32_low<false, false><<<grid, kThreads, 0, s>>>(a, v0, v1, nullptr, 32, off, edg);
      }
    }
  } else if (cls == MID) {
    k32_mid<<<cap_grid32((cnt + 7) / 8, sms * 8), kThreads, 0, s>>>(a, b, cnt);
  } else {
    k32_high<<<cap_grid32(cnt, sms * 4), 256, 0, s>>>(a, b, cnt);
  }
  return true;
}

void launch_refine_finalize64(const SolveArgs& a, cudaStream_t s) { k_refine_finalize64<<<1, 1, 0, s>>>(a.st); }

// Conditions of the refinement loop as one graph: the outer WHILE node runs
// FP64 residual sweeps while the solve is not done and under the cap (its
// bodies counted in graph_rounds, at most cap of them), the inner one the
// FP32 sweeps of a round until k_finalize32 ends the round.
__global__ void k_refine_arm(cudaGraphConditionalHandle h, State* st) {
  st->graph_rounds = 0;  // the dynamic modes' FP32 phase may have counted its own loop's bodies
  cudaGraphSetConditional(h, (!st->done && st->iter < st->max_iter) ? 1u : 0u);
}
__global__ void k_refine_arm_inner(cudaGraphConditionalHandle h, const State* st) {
  cudaGraphSetConditional(h, (!st->done && !st->inner_done) ? 1u : 0u);
}
__global__ void k_refine_cond(cudaGraphConditionalHandle h, State* st, int cap) {
  const int rounds = ++st->graph_rounds;
  cudaGraphSetConditional(h, (!st->done && st->iter < st->max_iter && rounds < cap) ? 1u : 0u);
}

void launch_refine_arm(cudaGraphConditionalHandle h, const SolveArgs& a, bool inner, cudaStream_t s) {
  if (inner) k_refine_arm_inner<<<1, 1, 0, s>>>(h, a.st);
  else k_refine_arm<<<1, 1, 0, s>>>(h, a.st);
}
void launch_refine_cond(cudaGraphConditionalHandle h, const SolveArgs& a, bool inner, int cap, cudaStream_t s) {
  if (inner) k_refine_arm_inner<<<1, 1, 0, s>>>(h, a.st);
  else k_refine_cond<<<1, 1, 0, s>>>(h, a.st, cap);
}

void launch_finalize32(const SolveArgs& a, cudaStream_t s) { k_finalize32<<<1, 1, 0, s>>>(a.st); }

void launch_refine_round0(const SolveArgs& a, int sms, cudaStream_t s) {
  k_refine_round0<<<cap_grid32((a.n + kThreads - 1) / kThreads, sms * 16), kThreads, 0, s>>>(a);
}

void launch_refine_commit(const SolveArgs& a, int sms, cudaStream_t s) {
  k_refine_commit<<<cap_grid32((a.n + kThreads - 1) / kThreads, sms * 16), kThreads, 0, s>>>(a);
}

}  // namespace prx
