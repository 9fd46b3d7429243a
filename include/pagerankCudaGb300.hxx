// pagerankCudaGb300.hxx -- the reference's C++ solver surface on the GB300 C ABI.
//
// Drop-in for the five templates of puzzlef/pagerank-cuda-dynamic
// inc/pagerankCuda.hxx:864-988, same names, template parameters and
// arguments:
//
//   pagerankStaticCuda<PARTITION, FLAG>(x, xt, o)
//   pagerankNaiveDynamicCuda<PARTITION, FLAG>(x, xt, q, o)
//   pagerankDynamicTraversalCuda<PARTITION, FLAG>(x, xt, y, yt, deletions, insertions, q, o)
//   pagerankDynamicFrontierCuda<PARTITION, FLAG>(x, xt, y, yt, deletions, insertions, q, o)
//   pagerankPruneDynamicFrontierCuda<PARTITION, FLAG>(x, xt, y, yt, deletions, insertions, q, o)
//
// G / H are any graph types with the reference DiGraph interface
// (key_type, span, order, size, empty, forEachVertexKey, forEachEdgeKey,
// degree, vertexValue; H's vertex value is the out-degree, as produced by
// transposeWithDegreeOmp, inc/transpose.hxx:128).  Like pagerankInvokeCuda
// (:713-849) each call renumbers the vertices densely in ascending id order
// (vertexKeys, inc/properties.hxx:26-33), uploads the CSRs, solves, and
// scatters the ranks back to a span-indexed vector; absent ids get 0.
// Ranks are computed in FP64; another V is converted on the way in and out.
// Errors throw std::runtime_error (the reference exits, inc/_cuda.hxx:136).
//
// PagerankOptions / PagerankResult (inc/pagerank.hxx:24-113) are defined
// here unless PRX_USE_REFERENCE_PAGERANK_TYPES is defined, for translation
// units that already include the reference's inc/pagerank.hxx.  Such a unit
// must not also include inc/pagerankCuda.hxx, which defines the same
// template names.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>
#include "pagerank_gb300.h"

#ifndef PRX_USE_REFERENCE_PAGERANK_TYPES
template <class V>
struct PagerankOptions {
  int repeat;
  V tolerance;
  V frontierTolerance;
  V pruneTolerance;
  V damping;
  int maxIterations;
  PagerankOptions(int repeat = 1, V tolerance = 1e-10, V frontierTolerance = 1e-6, V pruneTolerance = 1e-6,
                  V damping = 0.85, int maxIterations = 500)
      : repeat(repeat), tolerance(tolerance), frontierTolerance(frontierTolerance), pruneTolerance(pruneTolerance),
        damping(damping), maxIterations(maxIterations) {}
};

template <class V>
struct PagerankResult {
  std::vector<V> ranks;
  int iterations;
  float time;
  float initializationTime;
  float markingTime;
  float computationTime;
  PagerankResult() : ranks(), iterations(0), time(0), initializationTime(0), markingTime(0), computationTime(0) {}
  // inc/pagerank.hxx:98 (an rvalue vector) and :111 (an lvalue vector, moved from)
  PagerankResult(std::vector<V>&& ranks, int iterations = 0, float time = 0, float initializationTime = 0,
                 float markingTime = 0, float computationTime = 0)
      : ranks(std::move(ranks)), iterations(iterations), time(time), initializationTime(initializationTime),
        markingTime(markingTime), computationTime(computationTime) {}
  PagerankResult(std::vector<V>& ranks, int iterations = 0, float time = 0, float initializationTime = 0,
                 float markingTime = 0, float computationTime = 0)
      : ranks(std::move(ranks)), iterations(iterations), time(time), initializationTime(initializationTime),
        markingTime(markingTime), computationTime(computationTime) {}
};
#endif

namespace prx_cpp {

inline void check(int status, const char* where) {
  if (status != PRX_OK)
    throw std::runtime_error(std::string(where) + ": " + prx_status_string(status) + " (" + prx_last_error() + ")");
}

// One context per host thread on device 0 (the reference uses the current
// device and the legacy stream from a single thread).
struct ThreadContext {
  prx_context* c = nullptr;
  ~ThreadContext() {
    if (c) prx_context_destroy(c);
  }
};
inline prx_context* context() {
  static thread_local ThreadContext t;
  if (!t.c) check(prx_context_create(0, &t.c), "prx_context_create");
  return t.c;
}

// Dense CSR of a DiGraph over the vertex keys ks (ascending ids); 64-bit
// offsets, so graphs of 2^32 edges or more go through as well.
template <class G>
void csr_of(const G& x, const std::vector<uint32_t>& ks, const std::vector<uint32_t>& dense,
            std::vector<uint64_t>& off, std::vector<uint32_t>& edg) {
  off.clear();
  edg.clear();
  off.reserve(ks.size() + 1);
  uint64_t o = 0;
  for (uint32_t u : ks) {
    off.push_back(o);
    o += x.degree(u);
  }
  off.push_back(o);
  edg.reserve(o);
  for (uint32_t u : ks) x.forEachEdgeKey(u, [&](auto v) { edg.push_back(dense[v]); });
}

template <bool DYNAMIC, bool PARTITION, class G, class H, class K, class V>
PagerankResult<V> invoke(int mode, const G& y, const H& yt, const std::vector<std::tuple<K, K>>& deletions,
                         const std::vector<std::tuple<K, K>>& insertions, const std::vector<V>* q,
                         const PagerankOptions<V>& o) {
  const size_t S = yt.span();
  std::vector<uint32_t> ks, dense(S, UINT32_MAX);
  ks.reserve(yt.order());
  yt.forEachVertexKey([&](auto u) {
    dense[u] = (uint32_t)ks.size();
    ks.push_back((uint32_t)u);
  });
  const uint32_t N = (uint32_t)ks.size();
  std::vector<uint64_t> xoff, xtoff;
  std::vector<uint32_t> xedg, xtedg, xtdat(N);
  if (DYNAMIC) csr_of(y, ks, dense, xoff, xedg);
  csr_of(yt, ks, dense, xtoff, xtedg);
  for (uint32_t i = 0; i < N; ++i) xtdat[i] = (uint32_t)yt.vertexValue(ks[i]);
  std::vector<double> qc;
  if (q) {
    qc.resize(N);
    for (uint32_t i = 0; i < N; ++i) qc[i] = (double)(*q)[ks[i]];
  }
  std::vector<uint32_t> du, dv, iu, iv;
  for (const auto& e : deletions) { du.push_back(dense[std::get<0>(e)]); dv.push_back(dense[std::get<1>(e)]); }
  for (const auto& e : insertions) { iu.push_back(dense[std::get<0>(e)]); iv.push_back(dense[std::get<1>(e)]); }
  prx_context* ctx = context();
  prx_graph* g = nullptr;
  check(prx_graph_create64(ctx, N, xtedg.size(), DYNAMIC ? xoff.data() : nullptr, DYNAMIC ? xedg.data() : nullptr,
                           xtoff.data(), xtedg.data(), xtdat.data(), 0, 0, &g),
        "prx_graph_create64");
  prx_options po;
  prx_options_default(&po);
  po.repeat = o.repeat;
  po.tolerance = (double)o.tolerance;
  po.frontier_tolerance = (double)o.frontierTolerance;
  po.prune_tolerance = (double)o.pruneTolerance;
  po.damping = (double)o.damping;
  po.max_iterations = o.maxIterations;
  po.partition = PARTITION ? 1 : 0;
  std::vector<double> rc(N);
  prx_result res;
  const int st = prx_solve(ctx, g, mode, du.data(), dv.data(), du.size(), iu.data(), iv.data(), iu.size(),
                           q ? qc.data() : nullptr, &po, rc.data(), &res);
  prx_graph_destroy(g);
  check(st, "prx_solve");
  std::vector<V> r(S);
  for (uint32_t i = 0; i < N; ++i) r[ks[i]] = (V)rc[i];
  return PagerankResult<V>(r, res.iterations, res.time_ms, res.initialization_time_ms, res.marking_time_ms,
                           res.computation_time_ms);
}

}  // namespace prx_cpp

template <bool PARTITION = false, class FLAG = char, class G, class H, class V>
inline PagerankResult<V> pagerankStaticCuda(const G& x, const H& xt, const PagerankOptions<V>& o) {
  using K = typename G::key_type;
  if (xt.empty()) return {};
  return prx_cpp::invoke<false, PARTITION>(PRX_STATIC, x, xt, std::vector<std::tuple<K, K>>(),
                                           std::vector<std::tuple<K, K>>(), (const std::vector<V>*)nullptr, o);
}

template <bool PARTITION = false, class FLAG = char, class G, class H, class V>
inline PagerankResult<V> pagerankNaiveDynamicCuda(const G& x, const H& xt, const std::vector<V>* q,
                                                  const PagerankOptions<V>& o) {
  using K = typename G::key_type;
  if (xt.empty()) return {};
  return prx_cpp::invoke<false, PARTITION>(PRX_NAIVE_DYNAMIC, x, xt, std::vector<std::tuple<K, K>>(),
                                           std::vector<std::tuple<K, K>>(), q, o);
}

template <bool PARTITION = false, class FLAG = char, class G, class H, class K, class V>
inline PagerankResult<V> pagerankDynamicTraversalCuda(const G& x, const H& xt, const G& y, const H& yt,
                                                      const std::vector<std::tuple<K, K>>& deletions,
                                                      const std::vector<std::tuple<K, K>>& insertions,
                                                      const std::vector<V>* q, const PagerankOptions<V>& o) {
  if (xt.empty()) return {};
  return prx_cpp::invoke<true, PARTITION>(PRX_DYNAMIC_TRAVERSAL, y, yt, deletions, insertions, q, o);
}

template <bool PARTITION = false, class FLAG = char, class G, class H, class K, class V>
inline PagerankResult<V> pagerankDynamicFrontierCuda(const G& x, const H& xt, const G& y, const H& yt,
                                                     const std::vector<std::tuple<K, K>>& deletions,
                                                     const std::vector<std::tuple<K, K>>& insertions,
                                                     const std::vector<V>* q, const PagerankOptions<V>& o) {
  if (xt.empty()) return {};
  return prx_cpp::invoke<true, PARTITION>(PRX_DYNAMIC_FRONTIER, y, yt, deletions, insertions, q, o);
}

template <bool PARTITION = false, class FLAG = char, class G, class H, class K, class V>
inline PagerankResult<V> pagerankPruneDynamicFrontierCuda(const G& x, const H& xt, const G& y, const H& yt,
                                                          const std::vector<std::tuple<K, K>>& deletions,
                                                          const std::vector<std::tuple<K, K>>& insertions,
                                                          const std::vector<V>* q, const PagerankOptions<V>& o) {
  if (xt.empty()) return {};
  return prx_cpp::invoke<true, PARTITION>(PRX_PRUNE_DYNAMIC_FRONTIER, y, yt, deletions, insertions, q, o);
}
