// prx_device.cuh -- device helpers shared by the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "prx_internal.h"
#include "prx_softadd.h"

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

// GB300 executes two FP64 lanes per SM per clock, so one warp-wide FP64
// instruction costs as much pipe time as dozens of integer ones: the helpers
// below keep to the FP64 operations the reference's arithmetic needs and do
// conversions and comparisons on bit patterns.

// (double)d exactly, from integer operations: d = 2^e * 1.f with e the
// position of the leading one.
__device__ __forceinline__ double u32_to_f64(uint32_t d) {
  const uint32_t lz = __clz(d);  // 32 for d == 0
  const unsigned long long frac = ((unsigned long long)d << (21 + (lz & 31))) & ((1ull << 52) - 1);
  const unsigned long long bits = ((unsigned long long)(1054 - lz) << 52) | frac;  // 1023 + (31 - lz)
  return d ? __longlong_as_double((long long)bits) : 0.0;
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
  const double r = fma(-q, u32_to_f64(d), a);
  return fma(r, y, q);
}

// The relative-change tests of the frontier modes, RN(x / m) <= c and
// RN(x / m) > c with x = |a - b| and m = fmax(a, b).  For non-negative finite
// a, b (the ranks) m is the larger bit pattern, and non-negative doubles
// order as their bit patterns: away from a band of 64 ulps around RN(c*m)
// the exact quotient is more than an ulp of c from c (the product's rounding
// is one half ulp), so its rounding lies on the same side, and one FP64
// multiplication decides.  Inside the band, or for negative, infinite or NaN
// operands or a subnormal c*m, the quotient is formed as written.
struct RelChange {
  double x, m;
  bool fast;
};
__device__ __forceinline__ RelChange rel_change(double a, double b) {
  const long long ab = __double_as_longlong(a), bb = __double_as_longlong(b);
  RelChange r;
  r.x = fabs(a - b);
  r.fast = (ab | bb) >= 0 && __double_as_longlong(r.x) < 0x7ff0000000000000ll;
  r.m = r.fast ? __longlong_as_double(ab > bb ? ab : bb) : fmax(a, b);
  return r;
}
constexpr long long kRelBand = 64;
__device__ __forceinline__ int rel_side(const RelChange& r, double c) {  // -1 below c, +1 above, 0 undecided
  if (!r.fast) return 0;
  const long long xb = __double_as_longlong(r.x), cb = __double_as_longlong(c * r.m);
  if (cb < (1ll << 52)) return 0;  // c*m subnormal or zero
  return xb < cb - kRelBand ? -1 : (xb > cb + kRelBand ? 1 : 0);
}
__device__ __forceinline__ bool quot_le(const RelChange& r, double c) {
  const int side = rel_side(r, c);
  return side ? side < 0 : r.x / r.m <= c;
}
__device__ __forceinline__ bool quot_gt(const RelChange& r, double c) {
  const int side = rel_side(r, c);
  return side ? side > 0 : r.x / r.m > c;
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

// Edge id as stored in a layout: a hot source's number with the flag, else
// the id itself (hot_idx null: plain ids; see GraphDev::hot_idx, of a graph
// of `words` bitmap words).
__device__ __forceinline__ uint32_t layout_id(const uint32_t* __restrict__ hot_idx, uint32_t words, uint32_t u) {
  if (!hot_idx) return u;
  const uint32_t w = __ldg(hot_idx + (u >> 5)), below = w & ((1u << (u & 31u)) - 1u);
  return ((w >> (u & 31u)) & 1u) ? (kHotFlag | (__ldg(hot_idx + words + (u >> 5)) + __popc(below))) : u;
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

// acc + x for the whole warp (all lanes converged): with `alt`, and when
// every lane's operands are in add_nonneg_bits's range (sign clear, below
// 2^977: a warp-uniform test), on the integer pipes; otherwise a DADD.  The
// bits are the same either way.
__device__ __forceinline__ double add_alt(double acc, double x, bool alt) {
  if (alt) {
    const uint32_t ha = (uint32_t)__double2hiint(acc), hx = (uint32_t)__double2hiint(x);
    if (__all_sync(0xffffffffu, (ha > hx ? ha : hx) < kSoftAddHiLimit))
      return __longlong_as_double((long long)add_nonneg_bits((uint64_t)__double_as_longlong(acc),
                                                             (uint64_t)__double_as_longlong(x)));
  }
  return acc + x;
}

// FP64 row sums, one row per lane, for a whole warp: every lane calls it
// (lanes with nothing to add pass s == e).  Each lane adds c[edg[j]] for j in
// [s, e) onto acc front to back, as lane_row_sum does, but the warp issues
// exactly L adds, L the longest row: lane_row_sum's aligned head and tail
// groups take up to three predicated adds each, and predicated-off FP64
// instructions cost the warp as much as live ones.  Step k reads ids
// s+4k .. s+4k+3 out of the two aligned 16-byte groups they span (the lane's
// offset s & 3 picks them); a lane past its row's end adds +0.0, which leaves
// acc (a sum of non-negative terms from +0) unchanged.  int_adds (0 .. 4)
// of every four adds of a full step run on the integer pipes (add_alt), so
// the FP64 pipe, the sweep's bound, carries fewer of them.
__device__ __forceinline__ double warp_row_sums(const double* __restrict__ c, const uint32_t* __restrict__ edg,
                                                uint32_t s, uint32_t e, double acc,
                                                const double* __restrict__ ch, bool hot, uint32_t int_adds) {
  const uint32_t len = e - s;
  const uint32_t L = __reduce_max_sync(0xffffffffu, len);
  if (L == 0) return acc;
  const uint32_t j0 = s & ~3u, o = s & 3u;
  const uint4 z = make_uint4(0, 0, 0, 0);
  uint4 g0 = len ? __ldg(reinterpret_cast<const uint4*>(edg + j0)) : z;
  for (uint32_t t = 0; t < L; t += 4) {
    const uint32_t jn = j0 + t + 4;
    const uint4 g1 = jn < e ? __ldg(reinterpret_cast<const uint4*>(edg + jn)) : z;
    // ids at s+t+i, i < 4: the 8 words of g0:g1 shifted by o
    const bool o1 = o & 1u, o2 = o & 2u;
    const uint32_t a0 = o1 ? g0.y : g0.x, a1 = o1 ? g0.z : g0.y, a2 = o1 ? g0.w : g0.z, a3 = o1 ? g1.x : g0.w,
                   a4 = o1 ? g1.y : g1.x, a5 = o1 ? g1.z : g1.y;
    const uint32_t u0 = o2 ? a2 : a0, u1 = o2 ? a3 : a1, u2 = o2 ? a4 : a2, u3 = o2 ? a5 : a3;
    double x0 = t < len ? gather(c, ch, hot, u0) : 0.0;
    double x1 = t + 1 < len ? gather(c, ch, hot, u1) : 0.0;
    double x2 = t + 2 < len ? gather(c, ch, hot, u2) : 0.0;
    const double x3 = t + 3 < len ? gather(c, ch, hot, u3) : 0.0;
    if (t + 4 <= L) {
      acc = add_alt(acc, x0, int_adds >= 4);
      acc = add_alt(acc, x1, int_adds >= 2);
      acc = add_alt(acc, x2, int_adds >= 3);
      acc = add_alt(acc, x3, int_adds >= 1);
    } else {  // the last 1..3 adds; the trip count is the same in every lane
      for (uint32_t r = L - t; r; --r) {
        acc += x0;
        x0 = x1;
        x1 = x2;
      }
    }
    g0 = g1;
  }
  return acc;
}

}  // namespace prx
