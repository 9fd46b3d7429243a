// prx_host.cpp -- host-side graph utilities of the C ABI (no device work).
//
// Synthetic graph generators, batch generation / tidying, host batch apply
// and transpose.  All randomness comes from a counter-based hash
// (splitmix64's finaliser over (seed, stream, index)), so every output is a
// pure function of the arguments, independent of the thread count.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <omp.h>
#include "pagerank_gb300.h"
#include "prx_hash.h"

namespace {

using prx_hash::below;
using prx_hash::mix64;
using prx_hash::rnd;
inline double u01(uint64_t x) { return (double)(x >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)

template <class T>
T* xmalloc(size_t cnt) {
  return (T*)std::malloc(sizeof(T) * (cnt ? cnt : 1));
}

// Exclusive scan of cnt[0..n) into off[0..n] (serial: n is a vertex count).
void scan_offsets(const std::vector<uint64_t>& cnt, uint32_t n, std::vector<uint64_t>& off) {
  off.assign((size_t)n + 1, 0);
  for (uint32_t v = 0; v < n; ++v) off[v + 1] = off[v] + cnt[v];
}

// Sort + dedup each row of a CSR held as 64-bit offsets into a scratch array,
// then compact into a prx_host_csr with 32-bit offsets.
int finish_rows(uint32_t n, const std::vector<uint64_t>& off, uint32_t* scratch, prx_host_csr* out) {
  std::vector<uint64_t> keep((size_t)n, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    uint32_t* b = scratch + off[u];
    uint32_t* e = scratch + off[u + 1];
    std::sort(b, e);
    keep[u] = (uint64_t)(std::unique(b, e) - b);
  }
  std::vector<uint64_t> noff;
  scan_offsets(keep, n, noff);
  if (noff[n] > 0xffffffffull) return PRX_ERANGE;
  out->n = n;
  out->m = noff[n];
  out->off = xmalloc<uint32_t>((size_t)n + 1);
  out->edg = xmalloc<uint32_t>(noff[n]);
  if (!out->off || !out->edg) return PRX_ENOMEM;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    out->off[u] = (uint32_t)noff[u];
    std::memcpy(out->edg + noff[u], scratch + off[u], sizeof(uint32_t) * keep[u]);
  }
  out->off[n] = (uint32_t)noff[n];
  return PRX_OK;
}

// Build a CSR from `E` generated edges (edge(i) -> (u, v)) plus a self-loop on
// every vertex: count, scatter, then sort + dedup the rows.
template <class F>
int csr_from_edges(uint32_t n, uint64_t E, F edge, prx_host_csr* out) {
  std::vector<uint64_t> cnt((size_t)n, 1);  // the self-loop
  {
    std::vector<std::atomic<uint64_t>> c((size_t)n);
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < (int64_t)n; ++v) c[v].store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)E; ++i) {
      uint32_t u, v;
      edge((uint64_t)i, u, v);
      c[u].fetch_add(1, std::memory_order_relaxed);
    }
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < (int64_t)n; ++v) cnt[v] += c[v].load(std::memory_order_relaxed);
  }
  std::vector<uint64_t> off;
  scan_offsets(cnt, n, off);
  uint32_t* scratch = xmalloc<uint32_t>(off[n]);
  if (!scratch) return PRX_ENOMEM;
  {
    std::vector<std::atomic<uint64_t>> fill((size_t)n);
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
      scratch[off[v]] = (uint32_t)v;
      fill[v].store(off[v] + 1, std::memory_order_relaxed);
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)E; ++i) {
      uint32_t u, v;
      edge((uint64_t)i, u, v);
      scratch[fill[u].fetch_add(1, std::memory_order_relaxed)] = v;
    }
  }
  const int st = finish_rows(n, off, scratch, out);
  std::free(scratch);
  return st;
}

bool row_has(const prx_host_csr* x, uint32_t u, uint32_t v) {
  const uint32_t* b = x->edg + x->off[u];
  const uint32_t* e = x->edg + x->off[u + 1];
  return std::binary_search(b, e, v);
}

}  // namespace

extern "C" {

void prx_host_csr_free(prx_host_csr* g) {
  if (!g) return;
  std::free(g->off);
  std::free(g->edg);
  g->off = g->edg = nullptr;
  g->n = 0;
  g->m = 0;
}

void prx_host_free(void* p) { std::free(p); }

int prx_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, prx_host_csr* out) {
  if (!out || scale < 1 || scale > 31 || edge_factor < 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1)
    return PRX_EINVAL;
  std::memset(out, 0, sizeof(*out));
  const uint32_t n = 1u << scale;
  const uint64_t E = (uint64_t)edge_factor * n;
  // quadrant thresholds on 32 random bits per level (integer compares only)
  const uint64_t ta = (uint64_t)std::llround(a * 4294967296.0);
  const uint64_t tab = (uint64_t)std::llround((a + b) * 4294967296.0);
  const uint64_t tabc = (uint64_t)std::llround((a + b + c) * 4294967296.0);
  const uint64_t words = (uint64_t)(scale + 1) / 2;
  auto edge = [&](uint64_t i, uint32_t& u, uint32_t& v) {
    uint32_t uu = 0, vv = 0;
    uint64_t bits = 0;
    for (int l = 0; l < scale; ++l) {
      if ((l & 1) == 0) bits = rnd(seed, 1, i * words + (uint64_t)(l >> 1));
      const uint64_t r = (l & 1) ? (bits >> 32) : (bits & 0xffffffffull);
      const uint32_t ub = r >= tab;
      const uint32_t vb = (r >= ta && r < tab) || r >= tabc;
      uu = (uu << 1) | ub;
      vv = (vv << 1) | vb;
    }
    u = uu;
    v = vv;
  };
  return csr_from_edges(n, E, edge, out);
}

int prx_gen_weblike(uint32_t n, double alpha, double dmin, uint32_t dmax, double local, uint32_t window,
                    uint64_t seed, prx_host_csr* out) {
  if (!out || n == 0 || alpha <= 1 || dmin <= 0 || dmax == 0 || local < 0 || local > 1) return PRX_EINVAL;
  std::memset(out, 0, sizeof(*out));
  const double ex = -1.0 / (alpha - 1.0);
  const uint64_t tlocal = (uint64_t)std::llround(local * 4294967296.0);
  std::vector<uint64_t> cap((size_t)n);
#pragma omp parallel for schedule(static)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    const double x = 1.0 - u01(rnd(seed, 2, (uint64_t)u));  // (0, 1]
    const double d = std::floor(dmin * std::pow(x, ex));
    cap[u] = 1 + (uint64_t)std::min<double>(d, (double)dmax);
  }
  std::vector<uint64_t> off;
  scan_offsets(cap, n, off);
  uint32_t* scratch = xmalloc<uint32_t>(off[n]);
  if (!scratch) return PRX_ENOMEM;
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    uint32_t* row = scratch + off[u];
    row[0] = (uint32_t)u;  // self-loop
    const uint64_t d = cap[u] - 1;
    for (uint64_t k = 0; k < d; ++k) {
      const uint64_t h = rnd(seed, 3, off[u] + k);
      uint32_t v;
      if ((h & 0xffffffffull) < tlocal) {
        // within +/-window of u, wrapping around the id range
        const int64_t w = (int64_t)u - (int64_t)window + (int64_t)below(h, 2ull * window + 1);
        v = (uint32_t)(((w % (int64_t)n) + (int64_t)n) % (int64_t)n);
      } else {
        v = below(mix64(h), n);
      }
      row[1 + k] = v;
    }
  }
  const int st = finish_rows(n, off, scratch, out);
  std::free(scratch);
  return st;
}

int prx_gen_grid(uint32_t w, double diag, uint64_t seed, prx_host_csr* out) {
  if (!out || w == 0 || (uint64_t)w * w > 0xffffffffull || diag < 0 || diag > 1) return PRX_EINVAL;
  std::memset(out, 0, sizeof(*out));
  const uint32_t n = w * w;
  const uint64_t tdiag = (uint64_t)std::llround(diag * 4294967296.0);
  // edge slots: 4 neighbour slots per vertex + 2 diagonal slots per vertex;
  // slots that do not apply become self-loops (removed by the dedup).
  const uint64_t E = 6ull * n;
  auto edge = [&](uint64_t i, uint32_t& u, uint32_t& v) {
    const uint32_t x = (uint32_t)(i / 6), k = (uint32_t)(i % 6);
    const uint32_t r = x / w, c = x % w;
    u = v = x;
    if (k < 4) {
      static const int dr[4] = {0, 0, 1, -1}, dc[4] = {1, -1, 0, 0};
      const int64_t rr = (int64_t)r + dr[k], cc = (int64_t)c + dc[k];
      if (rr >= 0 && rr < w && cc >= 0 && cc < w) v = (uint32_t)(rr * w + cc);
      return;
    }
    const uint64_t h = rnd(seed, 4, x);
    if ((h & 0xffffffffull) >= tdiag) return;
    const uint32_t dir = (uint32_t)((h >> 32) & 3);
    const int64_t rr = (int64_t)r + ((dir & 1) ? 1 : -1), cc = (int64_t)c + ((dir & 2) ? 1 : -1);
    if (rr < 0 || rr >= w || cc < 0 || cc >= w) return;
    const uint32_t y = (uint32_t)(rr * w + cc);
    if (k == 4) v = y;  // x -> y
    else { u = y; v = x; }  // y -> x
  };
  return csr_from_edges(n, E, edge, out);
}

int prx_host_tidy_batch(const prx_host_csr* x, uint32_t* du, uint32_t* dv, uint64_t* nd, uint32_t* iu,
                        uint32_t* iv, uint64_t* ni) {
  // tidyBatchUpdateU (inc/batch.hxx:200-208): keep deletions that exist and
  // insertions that do not, sort by (u, v), drop duplicates.
  if (!x || !nd || !ni) return PRX_EINVAL;
  auto tidy = [&](uint32_t* u, uint32_t* v, uint64_t* len, bool exists) {
    std::vector<uint64_t> k;
    k.reserve(*len);
    for (uint64_t i = 0; i < *len; ++i) {
      if (u[i] >= x->n || v[i] >= x->n) continue;  // ids outside the graph are dropped
      if (row_has(x, u[i], v[i]) == exists) k.push_back(((uint64_t)u[i] << 32) | v[i]);
    }
    std::sort(k.begin(), k.end());
    k.erase(std::unique(k.begin(), k.end()), k.end());
    for (size_t i = 0; i < k.size(); ++i) {
      u[i] = (uint32_t)(k[i] >> 32);
      v[i] = (uint32_t)k[i];
    }
    *len = k.size();
  };
  tidy(du, dv, nd, true);
  tidy(iu, iv, ni, false);
  return PRX_OK;
}

int prx_gen_batch(const prx_host_csr* x, uint64_t nd_req, uint64_t ni_req, uint64_t seed, uint32_t** du,
                  uint32_t** dv, uint64_t* nd, uint32_t** iu, uint32_t** iv, uint64_t* ni) {
  if (!x || !du || !dv || !nd || !iu || !iv || !ni || x->n == 0) return PRX_EINVAL;
  const uint32_t n = x->n;
  const uint64_t m = x->m;
  *du = xmalloc<uint32_t>(nd_req);
  *dv = xmalloc<uint32_t>(nd_req);
  *iu = xmalloc<uint32_t>(ni_req);
  *iv = xmalloc<uint32_t>(ni_req);
  if (!*du || !*dv || !*iu || !*iv) return PRX_ENOMEM;
  std::vector<uint8_t> ok(nd_req, 0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)nd_req; ++i) {
    // a uniformly chosen existing edge; self-loops are kept (no dead ends)
    for (uint64_t t = 0; t < prx_hash::kDelTries && m; ++t) {
      const uint64_t e = ((rnd(seed, prx_hash::kDelStream, (uint64_t)i * prx_hash::kDelTries + t) >> 11) % m);
      const uint32_t u = (uint32_t)(std::upper_bound(x->off, x->off + n + 1, (uint32_t)e) - x->off - 1);
      const uint32_t v = x->edg[e];
      if (u == v) continue;
      (*du)[i] = u;
      (*dv)[i] = v;
      ok[i] = 1;
      break;
    }
  }
  uint64_t k = 0;
  for (uint64_t i = 0; i < nd_req; ++i)
    if (ok[i]) { (*du)[k] = (*du)[i]; (*dv)[k] = (*dv)[i]; ++k; }
  *nd = k;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)ni_req; ++i) {
    const uint64_t h = rnd(seed, prx_hash::kInsStream, (uint64_t)i);
    (*iu)[i] = below(h, n);
    (*iv)[i] = below(mix64(h), n);
  }
  *ni = ni_req;
  return prx_host_tidy_batch(x, *du, *dv, nd, *iu, *iv, ni);
}

int prx_host_apply_batch(const prx_host_csr* x, const uint32_t* du, const uint32_t* dv, uint64_t nd,
                         const uint32_t* iu, const uint32_t* iv, uint64_t ni, prx_host_csr* y) {
  // applyBatchUpdateOmpU (inc/batch.hxx:239-247) on sorted rows.
  if (!x || !y) return PRX_EINVAL;
  std::memset(y, 0, sizeof(*y));
  const uint32_t n = x->n;
  std::vector<uint64_t> dlo((size_t)n + 1), ilo((size_t)n + 1);
  for (uint32_t u = 0, i = 0; u <= n; ++u) { while (i < nd && du[i] < u) ++i; dlo[u] = i; }
  for (uint32_t u = 0, i = 0; u <= n; ++u) { while (i < ni && iu[i] < u) ++i; ilo[u] = i; }
  std::vector<uint64_t> deg((size_t)n);
#pragma omp parallel for schedule(static)
  for (int64_t u = 0; u < (int64_t)n; ++u)
    deg[u] = (uint64_t)(x->off[u + 1] - x->off[u]) - (dlo[u + 1] - dlo[u]) + (ilo[u + 1] - ilo[u]);
  std::vector<uint64_t> off;
  scan_offsets(deg, n, off);
  if (off[n] > 0xffffffffull) return PRX_ERANGE;
  y->n = n;
  y->m = off[n];
  y->off = xmalloc<uint32_t>((size_t)n + 1);
  y->edg = xmalloc<uint32_t>(off[n]);
  if (!y->off || !y->edg) return PRX_ENOMEM;
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    y->off[u] = (uint32_t)off[u];
    uint64_t i = x->off[u], e = x->off[u + 1], d = dlo[u], a = ilo[u], k = off[u];
    for (;;) {
      const bool ho = i < e, hi = a < ilo[u + 1];
      if (!ho && !hi) break;
      if (ho && (!hi || x->edg[i] < iv[a])) {
        const uint32_t w = x->edg[i++];
        while (d < dlo[u + 1] && dv[d] < w) ++d;
        if (d < dlo[u + 1] && dv[d] == w) { ++d; continue; }
        y->edg[k++] = w;
      } else if (ho && x->edg[i] == iv[a]) {
        y->edg[k++] = x->edg[i++];
        ++a;
      } else {
        y->edg[k++] = iv[a++];
      }
    }
  }
  y->off[n] = (uint32_t)off[n];
  return PRX_OK;
}

int prx_host_transpose(const prx_host_csr* x, prx_host_csr* xt, uint32_t* xtdat) {
  // transposeWithDegreeOmp (inc/transpose.hxx:110-134): in-edge rows with
  // sources ascending; vertex value = out-degree.
  if (!x || !xt || (!xtdat && x->n)) return PRX_EINVAL;
  std::memset(xt, 0, sizeof(*xt));
  const uint32_t n = x->n;
  std::vector<std::atomic<uint32_t>> c((size_t)n);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; ++v) c[v].store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u) {
    xtdat[u] = x->off[u + 1] - x->off[u];
    for (uint64_t i = x->off[u]; i < x->off[u + 1]; ++i) c[x->edg[i]].fetch_add(1, std::memory_order_relaxed);
  }
  xt->n = n;
  xt->m = x->m;
  xt->off = xmalloc<uint32_t>((size_t)n + 1);
  xt->edg = xmalloc<uint32_t>(x->m);
  if (!xt->off || !xt->edg) return PRX_ENOMEM;
  uint64_t run = 0;
  for (uint32_t v = 0; v < n; ++v) {
    xt->off[v] = (uint32_t)run;
    run += c[v].load(std::memory_order_relaxed);
    c[v].store(xt->off[v], std::memory_order_relaxed);
  }
  xt->off[n] = (uint32_t)run;
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < (int64_t)n; ++u)
    for (uint64_t i = x->off[u]; i < x->off[u + 1]; ++i)
      xt->edg[c[x->edg[i]].fetch_add(1, std::memory_order_relaxed)] = (uint32_t)u;
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t v = 0; v < (int64_t)n; ++v) std::sort(xt->edg + xt->off[v], xt->edg + xt->off[v + 1]);
  return PRX_OK;
}

}  // extern "C"
