// prx_tune.cu -- autotuner for the execution parameters that do not change
// results: the MID / HIGH in-degree boundary (warp or block per vertex, both
// in the reference's 256-way order), the source-chunk widths of the FP64
// and FP32 sweeps of the in-degree <= 64 rows, and the L2 fetch granularity
// (how much of a line a missed gather brings in: more helps when nearby
// contributions are read soon after, less when gathers are scattered), and
// how many of every four edge additions of the FP64 sweep run on the integer
// pipes (the FP64 pipe is the sweep's bound; the integer adder costs more
// instructions, so the balance depends on the graph).  No counterpart in the
// reference, which uses fixed thresholds (inc/pagerankCuda.hxx:625-638).
//
// Each candidate is timed by short solves on the graph itself (Static, 3
// iterations, FP64 or FP32 refinement, the default loop), best of two.  The
// picks are stored on the graph and cached per graph signature (n, m and the
// in-degree class sizes), in the process and optionally in a text file, so a
// graph of the same shape built again is tuned without trials.
#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include "prx_ctx.h"

namespace {

struct Pick {
  uint32_t mid_max, w64, w32;
  float ms64, ms32;
  int fetch;
  int int_adds;  // -1 none, 1 .. 4 (0: not tuned, e.g. a cache line without it)
};

std::mutex g_tune_mu;
std::map<std::string, Pick> g_tune_cache;

std::string signature(const GraphDev& g) {
  char buf[160];
  snprintf(buf, sizeof buf, "n%u_m%llu_low%u_%llu", g.n, (unsigned long long)g.m, g.cls_begin[1] - g.cls_begin[0],
           (unsigned long long)g.cls_edges[LOW]);
  return buf;
}

void load_file(const char* path) {
  if (!path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  char line[320], key[160];
  while (fgets(line, sizeof line, f)) {
    Pick p{};
    if (sscanf(line, "%159s %u %u %u %f %f %d %d", key, &p.mid_max, &p.w64, &p.w32, &p.ms64, &p.ms32, &p.fetch,
               &p.int_adds) >= 6)
      g_tune_cache[key] = p;
  }
  fclose(f);
}

void save_file(const char* path) {
  if (!path) return;
  FILE* f = fopen(path, "w");
  if (!f) return;
  for (const auto& kv : g_tune_cache)
    fprintf(f, "%s %u %u %u %.4f %.4f %d %d\n", kv.first.c_str(), kv.second.mid_max, kv.second.w64, kv.second.w32,
            kv.second.ms64, kv.second.ms32, kv.second.fetch, kv.second.int_adds);
  fclose(f);
}

// ms per iteration of a short Static solve (best of two), or < 0 on error.
float trial(prx_context* c, prx_graph* gr, double* ranks, int precision, uint32_t width, int* status,
            int fetch = -1, int int_adds = 0) {
  prx_options o;
  prx_options_default(&o);
  o.max_iterations = 3;
  o.precision = precision;
  o.chunk_vertices = width;
  o.l2_fetch_bytes = fetch;
  o.int_adds = int_adds;
  o.tolerance = 0.0;  // run all three iterations
  float best = -1.f;
  for (int rep = 0; rep < 2; ++rep) {
    prx_result r{};
    const int st = prx_solve_device(c, gr, PRX_STATIC, nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr, &o, ranks, &r);
    if (st) {
      *status = st;
      return -1.f;
    }
    const float ms = r.computation_time_ms / (r.iterations ? r.iterations : 1);
    if (best < 0 || ms < best) best = ms;
  }
  return best;
}

}  // namespace

cudaError_t prx::tune_apply_cached(GraphDev& g, int sms, cudaStream_t s) {
  if (g.n == 0) return cudaSuccess;
  Pick p;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const auto it = g_tune_cache.find(signature(g));
    if (it == g_tune_cache.end()) return cudaSuccess;
    p = it->second;
  }
  g.tuned_w64 = p.w64;
  g.tuned_w32 = p.w32;
  g.tuned_fetch = p.fetch;
  g.tuned_int_adds = p.int_adds;
  if (p.mid_max == g.mid_max) return cudaSuccess;
  // only the MID / HIGH lists depend on the boundary (not the LOW bitmap,
  // the reciprocals or source chunks, which a new graph does not have yet)
  g.mid_max = p.mid_max;
  return build_class_lists(g.xtoff, g.seg_shift, g.n, g.mid_max, g.cls_list, g.cls_begin, g.cls_edges, sms, s);
}

extern "C" {

int prx_autotune(prx_context* c, prx_graph* gr, const char* cache_path, prx_tune_result* out) {
  if (!c || !gr || gr->ctx != c) FAIL(PRX_EINVAL, "prx_autotune: bad context or graph");
  GraphDev& g = gr->g;
  prx_tune_result res{};
  res.mid_max = g.mid_max;
  if (g.n == 0) {
    if (out) *out = res;
    return PRX_OK;
  }
  TRY_CUDA_ST(cudaSetDevice(c->device));
  std::lock_guard<std::mutex> lock(g_tune_mu);
  load_file(cache_path);
  const std::string key = signature(g);
  auto it = g_tune_cache.find(key);
  if (it != g_tune_cache.end()) {
    const Pick& p = it->second;
    if (p.mid_max != g.mid_max) {
      g.mid_max = p.mid_max;
      TRY_CUDA_ST(build_classes(g, c->sms, c->stream));
      TRY_CUDA_ST(cudaStreamSynchronize(c->stream));
    }
    g.tuned_w64 = p.w64;
    g.tuned_w32 = p.w32;
    g.tuned_fetch = p.fetch;
    g.tuned_int_adds = p.int_adds;
    res = {p.mid_max, p.w64, p.w32, p.ms64, p.ms32, 0, 1, p.fetch, p.int_adds};
    if (out) *out = res;
    return PRX_OK;
  }
  double* ranks = nullptr;
  TRY_CUDA_ST(cudaMalloc(&ranks, sizeof(double) * g.n));
  int st = PRX_OK, trials = 0;
  g.tuned_int_adds = 0;  // steps 1-3 time with the library default
  // 1. MID / HIGH boundary, with the default chunk widths
  const uint32_t mids[] = {1024u, 4096u, 16384u};
  uint32_t best_mid = g.mid_max;
  float best = -1.f;
  for (uint32_t mm : mids) {
    if (g.mid_max != mm) {
      g.mid_max = mm;
      if (build_classes(g, c->sms, c->stream) != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess) {
        st = PRX_ECUDA;
        break;
      }
    }
    const float ms = trial(c, gr, ranks, PRX_FP64, 0, &st);
    ++trials;
    if (st) break;
    if (best < 0 || ms < best) {
      best = ms;
      best_mid = mm;
    }
  }
  if (!st && g.mid_max != best_mid) {
    g.mid_max = best_mid;
    if (build_classes(g, c->sms, c->stream) != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
      st = PRX_ECUDA;
  }
  // 2. source-chunk widths: no chunking and chunks of 200, 128, 64 MB (FP64)
  //    or 96, 48, 24 MB (FP32) of contributions
  uint32_t w64 = 0, w32 = 0;
  float ms64 = -1.f, ms32 = -1.f;
  if (!st) {
    g.tuned_w64 = g.tuned_w32 = 0;
    const uint32_t c64[] = {g.n, (200u << 20) / 8, (128u << 20) / 8, (64u << 20) / 8};
    const uint32_t c32[] = {g.n, (96u << 20) / 4, (48u << 20) / 4, (24u << 20) / 4};
    for (int pass = 0; pass < 2 && !st; ++pass) {
      const uint32_t* cand = pass ? c32 : c64;
      float& bms = pass ? ms32 : ms64;
      uint32_t& bw = pass ? w32 : w64;
      for (int k = 0; k < 4; ++k) {
        const uint32_t w = cand[k];
        if (k > 0 && w >= g.n) continue;  // the same as no chunking
        const float ms = trial(c, gr, ranks, pass ? PRX_FP32_REFINE : PRX_FP64, w, &st);
        ++trials;
        if (st) break;
        if (bms < 0 || ms < bms) {
          bms = ms;
          bw = w;
        }
      }
    }
  }
  // 3. L2 fetch granularity with those picks, by FP64 plus FP32 time
  int fetch = 0;
  if (!st) {
    g.tuned_w64 = w64;
    g.tuned_w32 = w32;
    g.tuned_fetch = 0;
    float bsum = -1.f;
    for (int f : {32, 64, 128}) {
      const float a = trial(c, gr, ranks, PRX_FP64, 0, &st, f);
      const float b = st ? 0.f : trial(c, gr, ranks, PRX_FP32_REFINE, 0, &st, f);
      trials += 2;
      if (st) break;
      if (bsum < 0 || a + b < bsum) {
        bsum = a + b;
        fetch = f;
        ms64 = a;
        ms32 = b;
      }
    }
  }
  // 4. integer-pipe adds of the FP64 sweep (none, or one to four of every
  //    four) with those picks, by FP64 time
  int int_adds = -1;
  if (!st) {
    g.tuned_fetch = fetch;
    float b = -1.f;
    for (int k : {-1, 1, 2, 3, 4}) {
      const float a = trial(c, gr, ranks, PRX_FP64, 0, &st, 0, k);
      ++trials;
      if (st) break;
      if (b < 0 || a < b) {
        b = a;
        int_adds = k;
      }
    }
    if (!st) ms64 = b;
  }
  cudaFree(ranks);
  if (st) return st;
  g.tuned_w64 = w64;
  g.tuned_w32 = w32;
  g.tuned_fetch = fetch;
  g.tuned_int_adds = int_adds;
  g_tune_cache[key] = {g.mid_max, w64, w32, ms64, ms32, fetch, int_adds};
  save_file(cache_path);
  res = {g.mid_max, w64, w32, ms64, ms32, trials, 0, fetch, int_adds};
  if (out) *out = res;
  return PRX_OK;
}

}  // extern "C"
