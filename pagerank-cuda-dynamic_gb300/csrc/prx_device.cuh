// prx_device.cuh -- device helpers shared by the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "prx_internal.h"

namespace prx {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Row segments (see GraphDev): index of row v's begin in the offsets, and
// the start of its segment's edges.  shift 32 / base null: the plain CSR.
__device__ __forceinline__ uint64_t seg_index(uint32_t v, uint32_t shift) {
  return (uint64_t)v + ((uint64_t)v >> shift);
}
__device__ __forceinline__ const uint32_t* seg_edges(const uint32_t* edg, const unsigned long long* base, uint32_t shift,
                                                     uint32_t v) {
  return base ? edg + base[(uint64_t)v >> shift] : edg;
}
__device__ __forceinline__ uint32_t row_len(const uint32_t* __restrict__ off, uint32_t shift, uint32_t v) {
  const uint64_t i = seg_index(v, shift);
  return off[i + 1] - off[i];
}

// In-degree class of v (see kLowMax).
__device__ __forceinline__ int in_class(const uint32_t* __restrict__ xtoff, uint32_t shift, uint32_t v,
                                        uint32_t mid_max) {
  const uint32_t d = row_len(xtoff, shift, v);
  return d <= kLowMax ? LOW : (d <= mid_max ? MID : HIGH);
}

// Set bit v of a bitmap; true if this call changed it from 0 to 1.  Bits only
// go 0 -> 1 while marking kernels run, so a set bit seen by the plain load is
// final and the atomic can be skipped.
__device__ __forceinline__ bool test_and_set(uint32_t* bm, uint32_t v) {
  const uint32_t bit = 1u << (v & 31u);
  if (bm[v >> 5] & bit) return false;
  return !(atomicOr(&bm[v >> 5], bit) & bit);
}

__device__ __forceinline__ void clear_bit(uint32_t* bm, uint32_t v) {
  atomicAnd(&bm[v >> 5], ~(1u << (v & 31u)));
}

// Append v to list/cnt.  Lanes of the active set that append to the same
// counter share one atomicAdd (safe under divergence).
__device__ __forceinline__ void push(uint32_t* list, uint32_t* cnt, uint32_t v) {
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, (unsigned long long)(uintptr_t)cnt);
  const int leader = __ffs(peers) - 1;
  const unsigned lane = lane_id();
  uint32_t base = 0;
  if ((int)lane == leader) base = atomicAdd(cnt, (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  list[base + __popc(peers & ((1u << lane) - 1u))] = v;
}

// Block-wide max of a non-negative double given as its bit pattern (for
// x >= 0 the IEEE-754 bit patterns order like the values), folded into *dst
// with one atomicMax per block.  Every thread of the block must call it; the
// leading barrier lets calls follow one another (warp 0 may still be reading
// the shared slots of the previous call).
__device__ __forceinline__ void block_max_bits(unsigned long long x, unsigned long long* dst) {
  __shared__ unsigned long long smax[32];
  for (int o = 16; o; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, o);
    x = y > x ? y : x;
  }
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if (lane_id() == 0) smax[w] = x;
  __syncthreads();
  if (w == 0) {
    x = lane_id() < (blockDim.x >> 5) ? smax[lane_id()] : 0ull;
    for (int o = 16; o; o >>= 1) {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, o);
      x = y > x ? y : x;
    }
    if (lane_id() == 0 && x) atomicMax(dst, x);
  }
}

// The same for a non-negative float given as its bit pattern.
__device__ __forceinline__ void block_max_u32(unsigned int x, unsigned int* dst) {
  __shared__ unsigned int smax[32];
  for (int o = 16; o; o >>= 1) x = max(x, __shfl_xor_sync(0xffffffffu, x, o));
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if (lane_id() == 0) smax[w] = x;
  __syncthreads();
  if (w == 0) {
    x = lane_id() < (blockDim.x >> 5) ? smax[lane_id()] : 0u;
    for (int o = 16; o; o >>= 1) x = max(x, __shfl_xor_sync(0xffffffffu, x, o));
    if (lane_id() == 0 && x) atomicMax(dst, x);
  }
}

__device__ __forceinline__ void block_sum_u64(unsigned long long x, unsigned long long* dst) {
  __shared__ unsigned long long ssum[32];
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if (lane_id() == 0) ssum[w] = x;
  __syncthreads();
  if (w == 0) {
    x = lane_id() < (blockDim.x >> 5) ? ssum[lane_id()] : 0ull;
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane_id() == 0 && x) atomicAdd(dst, x);
  }
}

__device__ __forceinline__ unsigned long long dbits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}

// a / d correctly rounded, for an integer d >= 1 and y = RN(1/d), by
// Markstein's method (P. Markstein, "IA-64 and Elementary Functions", 2000):
// q = RN(a*y) is within one ulp of a/d, so r = a - q*d is exact in one fma,
// and RN(q + r*y) is the correctly rounded quotient.  Three FP64 operations
// instead of a full division; valid while nothing over- or underflows (ranks
// and contributions here are far from both).  Checked bit for bit against
// the IEEE division by prx_selftest.
__device__ __forceinline__ double div_count(double a, uint32_t d, double y) {
  const double q = a * y;
  const double r = fma(-q, (double)d, a);
  return fma(r, y, q);
}

// RN(x / m) <= c and RN(x / m) > c for x >= 0, m >= 0 -- the comparisons of
// a relative change with a tolerance -- decided by one multiplication unless
// x lies within 2^-48 of c*m, where the quotient is formed as written.  Away
// from that band the rounded quotient is on the same side of c as the exact
// one (the product's rounding is < 2^-52 relative), so the result always
// equals the comparison of the correctly rounded quotient, NaN (0/0)
// included.
__device__ __forceinline__ bool quot_le(double x, double m, double c) {
  const double cm = c * m;
  if (x < cm * (1.0 - 0x1p-48)) return true;
  if (x > cm * (1.0 + 0x1p-48)) return false;
  return x / m <= c;
}
__device__ __forceinline__ bool quot_gt(double x, double m, double c) {
  const double cm = c * m;
  if (x > cm * (1.0 + 0x1p-48)) return true;
  if (x < cm * (1.0 - 0x1p-48)) return false;
  return x / m > c;
}

// FP32 rounds of the refinement stop once the change they predict for their
// next sweep -- this sweep's change times the larger of its last two ratios
// to the sweep before (the observed rate of the Jacobi iteration) -- is below
// kPredictSafety times the tolerance: the FP64 residual sweep that follows
// measures about that next change, so it passes without the FP32 sweep that
// would only confirm it.  The FP64 test still decides convergence; a wrong
// prediction costs one more round, never accuracy.  prev / prev2: the
// changes of the two sweeps before (0: none yet).
constexpr float kPredictSafety = 0.8f;
__device__ __forceinline__ bool fp32_round_done(float change, float prev, float prev2, double tol) {
  if (!(prev > 0.f && prev2 > 0.f && change < prev && prev < prev2)) return false;
  const float rate = fmaxf(change / prev, prev / prev2);
  return change * rate < kPredictSafety * (float)tol;
}

// The contribution of edge id u: with `hot` (a layout whose hot sources are
// encoded, kHotFlag | number) from the dense hot copy ch, else c[u].
template <class T>
__device__ __forceinline__ T gather(const T* __restrict__ c, const T* __restrict__ ch, bool hot, uint32_t u) {
  return __ldg((hot && (u & kHotFlag)) ? ch + (u ^ kHotFlag) : c + u);
}

// Sum of c[edg[j]] for j in [s, e) added front to back onto acc.  The edge
// ids are read as aligned 16-byte groups of four (edg must be 16-byte
// aligned and allocated per edge_slots); ids outside [s, e) in the first and
// last group are loaded but neither gathered nor added.  Four gathers are in
// flight per group.  hot / ch: see gather().
template <class T>
__device__ __forceinline__ T lane_row_sum(const T* __restrict__ c, const uint32_t* __restrict__ edg, uint32_t s,
                                          uint32_t e, T acc, const T* __restrict__ ch = nullptr, bool hot = false) {
  if (s >= e) return acc;
  uint32_t j = s & ~3u;
  if (j < s) {  // head group: ids j+1 .. j+3 from s on
    const uint4 u = __ldg(reinterpret_cast<const uint4*>(edg + j));
    const bool b1 = s <= j + 1 && j + 1 < e, b2 = s <= j + 2 && j + 2 < e, b3 = j + 3 < e;
    const T c1 = b1 ? gather(c, ch, hot, u.y) : T(0), c2 = b2 ? gather(c, ch, hot, u.z) : T(0),
            c3 = b3 ? gather(c, ch, hot, u.w) : T(0);
    if (b1) acc += c1;
    if (b2) acc += c2;
    if (b3) acc += c3;
    j += 4;
  }
  for (; j + 4 <= e; j += 4) {
    const uint4 u = __ldg(reinterpret_cast<const uint4*>(edg + j));
    const T c0 = gather(c, ch, hot, u.x), c1 = gather(c, ch, hot, u.y), c2 = gather(c, ch, hot, u.z),
            c3 = gather(c, ch, hot, u.w);
    acc += c0; acc += c1; acc += c2; acc += c3;
  }
  if (j < e) {  // tail group: ids j .. e-1 (at most 3)
    const uint4 u = __ldg(reinterpret_cast<const uint4*>(edg + j));
    const bool b1 = j + 1 < e, b2 = j + 2 < e;
    const T c0 = gather(c, ch, hot, u.x), c1 = b1 ? gather(c, ch, hot, u.y) : T(0),
            c2 = b2 ? gather(c, ch, hot, u.z) : T(0);
    acc += c0;
    if (b1) acc += c1;
    if (b2) acc += c2;
  }
  return acc;
}

}  // namespace prx
