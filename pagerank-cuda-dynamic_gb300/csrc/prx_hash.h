// prx_hash.h -- the counter-based random numbers of the generators, shared by
// the host generators (prx_host.cpp) and the device batch generator
// (prx_tidy.cu) so both give the same values: splitmix64's finaliser over
// (seed, stream, index).  Integer arithmetic only.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define PRX_HD __host__ __device__ __forceinline__
#else
#define PRX_HD inline
#endif

namespace prx_hash {

PRX_HD uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
PRX_HD uint64_t rnd(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
}
// [0, n) for n < 2^32
PRX_HD uint32_t below(uint64_t x, uint64_t n) { return (uint32_t)(((x >> 32) * n) >> 32); }

// Random-batch streams: deletion i tries edges rnd(seed, kDelStream, i * kDelTries + t)
// until it finds one that is not a self-loop; insertion i is the pair drawn
// from rnd(seed, kInsStream, i).
constexpr uint64_t kDelStream = 5, kInsStream = 6, kDelTries = 32;

}  // namespace prx_hash
