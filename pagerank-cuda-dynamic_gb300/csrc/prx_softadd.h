// Correctly rounded FP64 addition of non-negative doubles in integer
// operations only (host and device).
//
// GB300 executes FP64 at 2 lanes per SM per clock, so a warp-wide DADD holds
// an SM's FP64 pipe for 16 cycles while its integer pipes run 64 lanes per
// clock.  The in-degree <= 64 sweep adds one contribution per edge in the
// reference's order and is bound by that FP64 pipe; moving part of the adds
// to the integer pipes keeps the order and the bits (IEEE 754 addition is a
// function of its two operands) and spreads the work over both.
//
// The method is the guard / round / sticky adder of IEEE 754 arithmetic
// (D. Goldberg, "What every computer scientist should know about
// floating-point arithmetic", ACM Computing Surveys 23(1), 1991, section 1.4):
// align the smaller significand to the larger one keeping three extra bits,
// the lowest the OR of every bit shifted past it; add; on a carry shift one
// more bit into the sticky one; round to nearest, ties to even.  For operands
// of one sign nothing cancels, so no normalisation beyond that carry is
// needed.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PRX_HD __host__ __device__ __forceinline__
#else
#define PRX_HD inline
#endif

namespace prx {

// add_nonneg_bits takes operands whose high words are below this: sign clear
// and biased exponent below 2000, i.e. values below 2^977.  A sum of up to
// 2^32 such terms stays below 2^1009, so no addition along a row overflows.
constexpr uint32_t kSoftAddHiLimit = 2000u << 20;

// Bits of RN(x + y) for the bit patterns x, y of two doubles whose high words
// are below kSoftAddHiLimit (zeros and subnormals included).
PRX_HD uint64_t add_nonneg_bits(uint64_t x, uint64_t y) {
  // non-negative doubles order as their bit patterns
  const uint64_t h = x > y ? x : y, l = x > y ? y : x;
  const uint32_t eh = (uint32_t)(h >> 52), el = (uint32_t)(l >> 52);
  // a subnormal has exponent 1 and no hidden bit
  const uint32_t Eh = eh > 1u ? eh : 1u, El = el > 1u ? el : 1u;
  // significands: the exponent field replaced by the hidden bit (1 if the
  // field was non-zero), then three guard bits below
  const uint64_t mh = (h - ((uint64_t)(Eh - 1u) << 52)) << 3;
  const uint64_t ml = (l - ((uint64_t)(El - 1u) << 52)) << 3;
  const uint32_t d = Eh - El;
  const uint32_t k = d < 63u ? d : 63u;  // ml < 2^56: a shift of 56 or more leaves only the sticky bit
  const uint64_t al = ml >> k;
  uint64_t s = mh + (al | (uint64_t)((al << k) != ml));  // < 2^57
  const uint32_t c = (uint32_t)(s >> 56);                // carry out of the significand
  s = (s >> c) | (s & (uint64_t)c);
  const uint64_t r = s >> 3;
  // round up when the three extra bits exceed one half, or equal it and r is odd
  const uint64_t q = r + ((((uint32_t)s & 7u) + ((uint32_t)r & 1u) + 3u) >> 3);
  // q carries the hidden bit at 52 (a rounding carry into bit 53 moves to the
  // next binade), so adding it to the exponent field minus one is the encoding
  return ((uint64_t)(Eh + c - 1u) << 52) + q;
}

}  // namespace prx
