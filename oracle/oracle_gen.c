/*
 * oracle_gen.c -- seeded synthetic inputs for the oracle side (TEST
 * INFRASTRUCTURE ONLY: the CPU reference arm and tests build their graphs
 * with these functions, so that they never load the product library).
 *
 * The graphs equal, edge for edge, those of the product's host generators:
 * the same counter-based hash (splitmix64's finaliser, Steele et al. 2014,
 * over (seed, stream, index)), the same draws per vertex and per edge slot,
 * rows sorted and deduplicated, one self-loop per vertex.  tests/
 * test_oracle_gen.py checks the equality on the CPU.
 *
 *   orc_gen_weblike()    power-law out-degree, host-local targets
 *   orc_transpose_omp()  the in-CSR with sources ascending and out-degrees,
 *                        as transposeWithDegreeOmp (inc/transpose.hxx:110-134)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>
#include "pagerank_oracle.h"

static uint64_t g_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static uint64_t g_rnd(uint64_t seed, uint64_t stream, uint64_t i) {
  return g_mix64(g_mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
}
/* uniform in [0, n) from the high 32 bits, n < 2^32 */
static uint32_t g_below(uint64_t x, uint64_t n) { return (uint32_t)(((x >> 32) * n) >> 32); }
/* [0, 1) from the high 53 bits */
static double g_u01(uint64_t x) { return (double)(x >> 11) * (1.0 / 9007199254740992.0); }

static int cmp_u32(const void* a, const void* b) {
  const uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return (x > y) - (x < y);
}

/* insertion sort for short rows, qsort beyond */
static void sort_row(uint32_t* b, uint64_t len) {
  if (len > 32) {
    qsort(b, (size_t)len, sizeof(uint32_t), cmp_u32);
    return;
  }
  for (uint64_t i = 1; i < len; ++i) {
    const uint32_t x = b[i];
    uint64_t j = i;
    while (j > 0 && b[j - 1] > x) { b[j] = b[j - 1]; --j; }
    b[j] = x;
  }
}

int orc_gen_weblike(uint32_t n, double alpha, double dmin, uint32_t dmax, double local,
                    uint32_t window, uint64_t seed, uint32_t** xoff_out, uint32_t** xedg_out,
                    uint64_t* m_out) {
  if (!xoff_out || !xedg_out || !m_out || n == 0 || alpha <= 1 || dmin <= 0 || dmax == 0 ||
      local < 0 || local > 1)
    return -1;
  *xoff_out = NULL;
  *xedg_out = NULL;
  *m_out = 0;
  const double ex = -1.0 / (alpha - 1.0);
  const uint64_t tlocal = (uint64_t)llround(local * 4294967296.0);
  uint64_t* off = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)n + 1));
  uint64_t* keep = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n);
  if (!off || !keep) { free(off); free(keep); return -2; }
  /* slots per vertex: 1 (self-loop) + min(floor(dmin * x^(-1/(alpha-1))), dmax) */
  #pragma omp parallel for schedule(static)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    const double x = 1.0 - g_u01(g_rnd(seed, 2, (uint64_t)u));  /* (0, 1] */
    const double d = floor(dmin * pow(x, ex));
    keep[u] = 1 + (uint64_t)(d < (double)dmax ? d : (double)dmax);
  }
  off[0] = 0;
  for (uint32_t u = 0; u < n; ++u) off[u + 1] = off[u] + keep[u];
  uint32_t* scratch = (uint32_t*)malloc(sizeof(uint32_t) * (off[n] ? off[n] : 1));
  if (!scratch) { free(off); free(keep); return -2; }
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    uint32_t* row = scratch + off[u];
    const uint64_t d = keep[u] - 1;
    row[0] = (uint32_t)u;
    for (uint64_t k = 0; k < d; ++k) {
      /* slot index off[u] + k draws one target: local (within +/-window,
       * wrapping) when the low 32 bits fall under `local`, else uniform */
      const uint64_t h = g_rnd(seed, 3, off[u] + k);
      uint32_t v;
      if ((h & 0xffffffffull) < tlocal) {
        const int64_t w = (int64_t)u - (int64_t)window + (int64_t)g_below(h, 2ull * window + 1);
        v = (uint32_t)(((w % (int64_t)n) + (int64_t)n) % (int64_t)n);
      } else {
        v = g_below(g_mix64(h), n);
      }
      row[1 + k] = v;
    }
    sort_row(row, d + 1);
    uint64_t w = 0;
    for (uint64_t i = 0; i <= d; ++i)
      if (i == 0 || row[i] != row[w - 1]) row[w++] = row[i];
    keep[u] = w;
  }
  uint64_t m = 0;
  for (uint32_t u = 0; u < n; ++u) m += keep[u];
  if (m > 0xffffffffull) { free(off); free(keep); free(scratch); return -3; }
  uint32_t* xoff = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
  uint32_t* xedg = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
  uint64_t* noff = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)n + 1));
  if (!xoff || !xedg || !noff) {
    free(off); free(keep); free(scratch); free(xoff); free(xedg); free(noff);
    return -2;
  }
  noff[0] = 0;
  for (uint32_t u = 0; u < n; ++u) noff[u + 1] = noff[u] + keep[u];
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    xoff[u] = (uint32_t)noff[u];
    memcpy(xedg + noff[u], scratch + off[u], sizeof(uint32_t) * keep[u]);
  }
  xoff[n] = (uint32_t)m;
  free(off); free(keep); free(scratch); free(noff);
  *xoff_out = xoff;
  *xedg_out = xedg;
  *m_out = m;
  return 0;
}

void orc_transpose_omp(uint32_t n, const uint32_t* xoff, const uint32_t* xedg,
                       uint32_t* xtoff, uint32_t* xtedg, uint32_t* xtdat) {
  /* in-degree counts with atomic adds, a serial scan, an atomic scatter, then
   * every in-row sorted: the same rows as the serial orc_transpose */
  uint32_t* cnt = (uint32_t*)calloc((size_t)n + 1, sizeof(uint32_t));
  if (!cnt) return;
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    xtdat[u] = xoff[u + 1] - xoff[u];
    for (uint64_t i = xoff[u]; i < xoff[u + 1]; ++i) {
      #pragma omp atomic
      cnt[xedg[i]]++;
    }
  }
  uint64_t run = 0;
  for (uint32_t v = 0; v < n; ++v) {
    xtoff[v] = (uint32_t)run;
    run += cnt[v];
    cnt[v] = xtoff[v];
  }
  xtoff[n] = (uint32_t)run;
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u)
    for (uint64_t i = xoff[u]; i < xoff[u + 1]; ++i) {
      uint32_t p;
      #pragma omp atomic capture
      p = cnt[xedg[i]]++;
      xtedg[p] = (uint32_t)u;
    }
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t v = 0; v < (int64_t)n; ++v) sort_row(xtedg + xtoff[v], (uint64_t)xtoff[v + 1] - xtoff[v]);
  free(cnt);
}

void orc_free(void* p) { free(p); }
