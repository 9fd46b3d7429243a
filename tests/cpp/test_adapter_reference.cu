// A translation unit shaped like the reference's main.cu, built against the
// reference's own headers: its DiGraph, batch, transpose and OpenMP PageRank
// code (inc/main.hxx's list minus inc/pagerankCuda.hxx), with the GB300
// adapter standing in for the CUDA solvers.  PRX_USE_REFERENCE_PAGERANK_TYPES
// makes the adapter use the reference's PagerankOptions / PagerankResult.
// The five solver templates are called as main.cu:93-139 calls them, on a
// DiGraph<uint32_t> with a self-loop on every vertex, and compared with the
// reference's pagerankStaticOmp (main.cu:65).  Compiled (and linked against
// the library) by tests/test_cpp_adapter.py where the reference's headers
// are present; it runs where a GPU is present too.
#define BUILD  0
#define OPENMP 1
#define CUDA   1
#include "_main.hxx"
#include "Graph.hxx"
#include "csr.hxx"
#include "properties.hxx"
#include "duplicate.hxx"
#include "transpose.hxx"
#include "selfLoop.hxx"
#include "batch.hxx"
#include "pagerank.hxx"
#include "pagerankPrune.hxx"
#define PRX_USE_REFERENCE_PAGERANK_TYPES
#include "pagerankCudaGb300.hxx"
#include <cstdio>
#include <tuple>
#include <vector>

using namespace std;

static uint64_t rng_state = 0x9E3779B97F4A7C15ull;
static uint32_t draw(uint32_t n) {
  rng_state ^= rng_state << 13; rng_state ^= rng_state >> 7; rng_state ^= rng_state << 17;
  return (uint32_t)(rng_state % n);
}

template <class V>
static double linf(const vector<V>& a, const vector<V>& b) {
  double e = 0;
  for (size_t i = 0; i < a.size() && i < b.size(); ++i) e = max(e, (double)abs(a[i] - b[i]));
  return a.size() == b.size() ? e : 1.0;
}

int main() {
  using K = uint32_t;
  using V = double;
  const K N = 4000;
  DiGraph<K> x;
  // ids 0, 2, 4, ...: absent odd ids exercise the dense renumbering and the
  // span-indexed results (absent ids get 0)
  for (K i = 0; i < 12 * N; ++i) x.addEdge(2 * draw(N), 2 * draw(N));
  x.update();
  auto fl = [](auto u) { return true; };
  x = addSelfLoopsOmp(x, None(), fl);
  auto xt = transposeWithDegreeOmp(x);
  vector<tuple<K, K>> deletions, insertions;
  for (K i = 0; i < 60; ++i) insertions.push_back({2 * draw(N), 2 * draw(N)});
  x.forEachVertexKey([&](auto u) {
    if (deletions.size() < 20 && x.degree(u) > 2) x.forEachEdgeKey(u, [&](auto v) {
      if (v != u && deletions.size() < 20) deletions.push_back({u, v});
    });
  });
  auto y = duplicate(x);
  tidyBatchUpdateU(deletions, insertions, y);
  applyBatchUpdateOmpU(y, deletions, insertions);
  auto yt = transposeWithDegreeOmp(y);
  const int repeat = 1;
  auto r0 = pagerankStaticOmp(xt, PagerankOptions<V>(1, 1e-100));
  auto s0 = pagerankStaticOmp(yt, PagerankOptions<V>(1, 1e-100));
  auto R = r0.ranks;
  int bad = 0;
  auto report = [&](const char* name, const PagerankResult<V>& a, const PagerankResult<V>& ref, double tol) {
    const double e = linf(a.ranks, ref.ranks);
    printf("%-40s %3d iter  linf %.3e  %s\n", name, a.iterations, e, e <= tol ? "ok" : "MISMATCH");
    bad += e > tol;
  };
  report("pagerankStaticCuda<false>", pagerankStaticCuda<false>(x, xt, PagerankOptions<V>(repeat)), r0, 5e-9);
  report("pagerankStaticCuda<true>", pagerankStaticCuda<true>(y, yt, PagerankOptions<V>(repeat)), s0, 5e-9);
  report("pagerankNaiveDynamicCuda<false>", pagerankNaiveDynamicCuda<false>(y, yt, &R, {repeat}), s0, 5e-9);
  report("pagerankDynamicTraversalCuda<false>",
         pagerankDynamicTraversalCuda<false>(x, xt, y, yt, deletions, insertions, &R, {repeat}), s0, 5e-9);
  report("pagerankDynamicFrontierCuda<false>",
         pagerankDynamicFrontierCuda<false>(x, xt, y, yt, deletions, insertions, &R, {repeat}), s0, 1e-6);
  report("pagerankPruneDynamicFrontierCuda<true>",
         pagerankPruneDynamicFrontierCuda<true>(x, xt, y, yt, deletions, insertions, &R, {repeat}), s0, 1e-6);
  // the rvalue constructor of PagerankResult (inc/pagerank.hxx:98)
  PagerankResult<V> moved(vector<V>(3, 1.0), 2);
  bad += moved.ranks.size() != 3 || moved.iterations != 2;
  DiGraph<K> empty;
  auto et = transposeWithDegreeOmp(empty);
  bad += !pagerankStaticCuda<false>(empty, et, PagerankOptions<V>(repeat)).ranks.empty();
  printf("%s\n", bad ? "FAILED" : "all ok");
  return bad ? 1 : 0;
}
