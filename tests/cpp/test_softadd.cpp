// Host check of prx::add_nonneg_bits against the FPU's IEEE 754 addition
// (round to nearest, ties to even) on seeded operands: uniform bit patterns,
// every exponent difference 0..70 with random and extreme significands,
// exact and near ties, carries out of the binade, zeros and subnormals,
// PageRank-like magnitudes, and long sequential sums.  Prints the mismatch
// count and exits non-zero on any mismatch.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "prx_softadd.h"

static uint64_t bits_of(double a) {
  uint64_t u;
  memcpy(&u, &a, 8);
  return u;
}
static double from_bits(uint64_t u) {
  double a;
  memcpy(&a, &u, 8);
  return a;
}

struct Rng {  // splitmix64
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
};

static const uint64_t M52 = (1ull << 52) - 1;
static long long checked = 0, bad = 0;

static void check(uint64_t x, uint64_t y) {
  // operands the kernels hand over: sign clear, high word below the limit
  if ((uint32_t)(x >> 32) >= prx::kSoftAddHiLimit || (uint32_t)(y >> 32) >= prx::kSoftAddHiLimit) return;
  const volatile double a = from_bits(x), b = from_bits(y);
  const uint64_t want = bits_of(a + b);
  const uint64_t got = prx::add_nonneg_bits(x, y);
  const uint64_t got2 = prx::add_nonneg_bits(y, x);
  ++checked;
  if (got != want || got2 != want) {
    if (bad < 10)
      printf("MISMATCH x=%016llx y=%016llx want=%016llx got=%016llx/%016llx\n", (unsigned long long)x,
             (unsigned long long)y, (unsigned long long)want, (unsigned long long)got, (unsigned long long)got2);
    ++bad;
  }
}

static uint64_t make(uint64_t e, uint64_t m) { return (e << 52) | (m & M52); }

static uint64_t mant(Rng& g) {
  switch (g.next() % 8) {
    case 0: return 0;
    case 1: return M52;
    case 2: return M52 - (g.next() % 8);
    case 3: return g.next() % 8;
    case 4: return (g.next() & M52) & ~7ull;
    case 5: return 1ull << (g.next() % 52);
    default: return g.next() & M52;
  }
}

int main(int argc, char** argv) {
  long long scale = argc > 1 ? atoll(argv[1]) : 1;
  Rng g{12345};
  // 1. uniform bit patterns below the limit
  for (long long i = 0; i < 4000000 * scale; ++i) check(g.next() % (2000ull << 52), g.next() % (2000ull << 52));
  // 2. every exponent difference 0..70, random and extreme significands,
  //    exponents across the range (subnormal and zero when the field is 0)
  for (long long i = 0; i < 8000000 * scale; ++i) {
    const uint64_t e1 = g.next() % 2000, dd = g.next() % 71;
    const uint64_t e2 = e1 >= dd ? e1 - dd : 0;
    check(make(e1, mant(g)), make(e2, mant(g)));
  }
  // 3. ties and near ties: y around half an ulp of x (and its neighbours)
  for (long long i = 0; i < 2000000 * scale; ++i) {
    const uint64_t e1 = 60 + g.next() % 1900;
    const uint64_t x = make(e1, mant(g));
    for (int sh = 52; sh <= 56; ++sh) {
      const uint64_t e2 = e1 - (uint64_t)sh;
      check(x, make(e2, 0));
      check(x, make(e2, 1));
      check(x, make(e2, M52));
      check(x, make(e2, g.next() & M52));
    }
  }
  // 4. carries: both operands near the top of one binade
  for (long long i = 0; i < 2000000 * scale; ++i) {
    const uint64_t e1 = 1 + g.next() % 1998;
    check(make(e1, M52 - (g.next() % 1024)), make(e1 - (g.next() % 3), M52 - (g.next() % 1024)));
  }
  // 5. zeros, subnormals, the smallest normals
  for (long long i = 0; i < 1000000 * scale; ++i) {
    const uint64_t a = g.next() % 4 == 0 ? 0 : (g.next() & M52);
    const uint64_t b = g.next() % 3 == 0 ? make(1 + g.next() % 3, g.next()) : (g.next() & M52);
    check(a, b);
    check(a, 0);
  }
  check(0, 0);
  // 6. PageRank-like magnitudes: contributions 1e-21 .. 1 added in sequence,
  //    both ways, the running sums compared at every step
  for (long long row = 0; row < 200000 * scale; ++row) {
    double acc = 0.0;
    uint64_t sacc = 0;
    const int len = 1 + (int)(g.next() % 200);
    for (int k = 0; k < len; ++k) {
      const double u = (double)(g.next() >> 11) * (1.0 / 9007199254740992.0);
      double t = u;
      for (int p = (int)(g.next() % 70); p > 0; --p) t *= 0.5;
      if (g.next() % 16 == 0) t = 0.0;
      check(bits_of(acc), bits_of(t));
      acc = acc + t;
      sacc = prx::add_nonneg_bits(sacc, bits_of(t));
      if (sacc != bits_of(acc)) {
        if (bad < 10) printf("MISMATCH in a sequential sum at row %lld step %d\n", row, k);
        ++bad;
        break;
      }
    }
  }
  printf("checked %lld sums, %lld mismatches\n", checked, bad);
  return bad ? 1 : 0;
}
