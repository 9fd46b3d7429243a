// Exercises include/pagerankCudaGb300.hxx the way the reference's main.cu
// calls inc/pagerankCuda.hxx: DiGraph-like inputs (non-contiguous vertex ids,
// so the dense renumbering and span-indexed scatter are exercised), the five
// solver templates, and a comparison with the oracle's GPU-semantics solve on
// the dense CSR.  Built and run by tests/test_cpp_adapter.py on a GPU.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <tuple>
#include <vector>
#include "pagerankCudaGb300.hxx"
#include "../../oracle/pagerank_oracle.h"

using K = uint32_t;

// Minimal DiGraph with the interface the adapter needs.
template <class V = int>
struct MiniGraph {
  using key_type = K;
  std::vector<bool> exists;
  std::vector<V> values;
  std::vector<std::vector<K>> edges;
  size_t N = 0, M = 0;
  size_t span() const { return exists.size(); }
  size_t order() const { return N; }
  size_t size() const { return M; }
  bool empty() const { return N == 0; }
  size_t degree(K u) const { return u < span() ? edges[u].size() : 0; }
  V vertexValue(K u) const { return u < span() ? values[u] : V(); }
  template <class F> void forEachVertexKey(F f) const { for (K u = 0; u < span(); ++u) if (exists[u]) f(u); }
  template <class F> void forEachEdgeKey(K u, F f) const { for (K v : edges[u]) f(v); }
  void addVertex(K u, V d = V()) {
    if (u >= span()) { exists.resize(u + 1); values.resize(u + 1); edges.resize(u + 1); }
    if (!exists[u]) { exists[u] = true; ++N; }
    values[u] = d;
  }
  void addEdge(K u, K v) { addVertex(u, values.size() > u ? values[u] : V()); addVertex(v, values.size() > v ? values[v] : V()); edges[u].push_back(v); }
  void update() {
    M = 0;
    for (auto& e : edges) { std::sort(e.begin(), e.end()); e.erase(std::unique(e.begin(), e.end()), e.end()); M += e.size(); }
  }
};

template <class G>
MiniGraph<K> transposeWithDegree(const G& x) {
  MiniGraph<K> a;
  x.forEachVertexKey([&](K u) { a.addVertex(u, (K)x.degree(u)); });
  x.forEachVertexKey([&](K u) { x.forEachEdgeKey(u, [&](K v) { a.edges[v].push_back(u); }); });
  a.update();
  return a;
}

static uint64_t rng_state = 88172645463325252ull;
static uint32_t rnd(uint32_t n) { rng_state ^= rng_state << 13; rng_state ^= rng_state >> 7; rng_state ^= rng_state << 17; return (uint32_t)(rng_state % n); }

int main() {
  // ids 0, 3, 6, ... exist (span 3*NV), every vertex has a self-loop
  const K NV = 3000;
  MiniGraph<> x;
  for (K i = 0; i < NV; ++i) x.addVertex(3 * i);
  for (K i = 0; i < NV; ++i) x.addEdge(3 * i, 3 * i);
  for (int e = 0; e < 40000; ++e) {
    K u = rnd(NV), v = rnd(NV);
    if (e % 7 == 0) v = 5;  // a hub with in-degree > 64
    x.addEdge(3 * u, 3 * v);
  }
  x.update();
  std::vector<std::tuple<K, K>> del, ins;
  MiniGraph<> y = x;
  for (int e = 0; e < 40; ++e) {
    K u = rnd(NV), v = rnd(NV);
    auto& row = y.edges[3 * u];
    if (!std::binary_search(row.begin(), row.end(), 3 * v)) { ins.push_back({3 * u, 3 * v}); row.push_back(3 * v); std::sort(row.begin(), row.end()); }
  }
  for (int e = 0; e < 10; ++e) {
    K u = 3 * rnd(NV);
    auto& row = y.edges[u];
    for (K v : row) if (v != u) { del.push_back({u, v}); row.erase(std::find(row.begin(), row.end(), v)); break; }
  }
  std::sort(ins.begin(), ins.end());
  ins.erase(std::unique(ins.begin(), ins.end()), ins.end());
  std::sort(del.begin(), del.end());
  del.erase(std::unique(del.begin(), del.end()), del.end());
  y.update();
  auto xt = transposeWithDegree(x);
  auto yt = transposeWithDegree(y);

  auto s0 = pagerankStaticCuda<false>(x, xt, PagerankOptions<double>());
  auto s1 = pagerankStaticCuda<true>(x, xt, PagerankOptions<double>());
  auto nd = pagerankNaiveDynamicCuda<false>(y, yt, &s0.ranks, PagerankOptions<double>());
  auto dt = pagerankDynamicTraversalCuda<false>(x, xt, y, yt, del, ins, &s0.ranks, PagerankOptions<double>());
  auto df = pagerankDynamicFrontierCuda<false>(x, xt, y, yt, del, ins, &s0.ranks, PagerankOptions<double>());
  auto dp = pagerankPruneDynamicFrontierCuda<true>(x, xt, y, yt, del, ins, &s0.ranks, PagerankOptions<double>());
  auto sf = pagerankStaticCuda<false>(x, xt, PagerankOptions<float>());

  // oracle on the dense CSR (ids / 3)
  auto dense = [&](const MiniGraph<>& g, std::vector<uint32_t>& off, std::vector<uint32_t>& edg) {
    off.assign(1, 0);
    edg.clear();
    g.forEachVertexKey([&](K u) { for (K v : g.edges[u]) edg.push_back(v / 3); off.push_back((uint32_t)edg.size()); });
  };
  std::vector<uint32_t> xo, xe, yo, ye;
  dense(x, xo, xe);
  dense(y, yo, ye);
  std::vector<uint32_t> xto(NV + 1), xte(xe.size()), xtd(NV), yto(NV + 1), yte(ye.size()), ytd(NV);
  orc_transpose(NV, xo.data(), xe.data(), xto.data(), xte.data(), xtd.data());
  orc_transpose(NV, yo.data(), ye.data(), yto.data(), yte.data(), ytd.data());
  std::vector<uint32_t> du, dv, iu, iv;
  for (auto& e : del) { du.push_back(std::get<0>(e) / 3); dv.push_back(std::get<1>(e) / 3); }
  for (auto& e : ins) { iu.push_back(std::get<0>(e) / 3); iv.push_back(std::get<1>(e) / 3); }
  orc_options o = {1e-10, 1e-6, 1e-6, 0.85, 500};
  std::vector<double> q(NV), want(NV);
  for (K i = 0; i < NV; ++i) q[i] = s0.ranks[3 * i];
  int fails = 0;
  auto cmp = [&](const char* name, int mode, const PagerankResult<double>& got, const double* qq, bool on_y) {
    const int it = orc_solve(mode, NV, on_y ? ye.size() : xe.size(), on_y ? yo.data() : xo.data(), on_y ? ye.data() : xe.data(),
                             on_y ? yto.data() : xto.data(), on_y ? yte.data() : xte.data(), on_y ? ytd.data() : xtd.data(),
                             du.data(), dv.data(), du.size(), iu.data(), iv.data(), iu.size(), qq, &o, want.data(), nullptr);
    const size_t S = x.span();  // ranks are indexed by original id, span = 3*(NV-1)+1
    bool ok = got.iterations == it && got.ranks.size() == S;
    for (K i = 0; ok && i < S; ++i) ok = (i % 3) ? got.ranks[i] == 0 : got.ranks[i] == want[i / 3];
    printf("%-28s iterations %3d (oracle %3d) %s\n", name, got.iterations, it, ok ? "bit-exact" : "MISMATCH");
    fails += !ok;
  };
  cmp("pagerankStaticCuda<false>", 0, s0, nullptr, false);
  cmp("pagerankStaticCuda<true>", 0, s1, nullptr, false);
  cmp("pagerankNaiveDynamicCuda", 1, nd, q.data(), true);
  cmp("pagerankDynamicTraversalCuda", 2, dt, q.data(), true);
  cmp("pagerankDynamicFrontierCuda", 3, df, q.data(), true);
  cmp("pagerankPruneDynamicFrontier", 4, dp, q.data(), true);
  // PagerankOptions<float> carries float-rounded parameters (damping
  // 0.85f = 0.8500000238...), so the solve differs slightly from the FP64 one.
  bool fok = sf.ranks.size() == s0.ranks.size();
  for (K i = 0; fok && i < s0.ranks.size(); ++i) fok = std::fabs(sf.ranks[i] - s0.ranks[i]) <= 1e-5 * s0.ranks[i] + 1e-12;
  printf("%-28s %s\n", "V=float", fok ? "ok" : "MISMATCH");
  fails += !fok;
  MiniGraph<> e0;
  auto emp = pagerankStaticCuda<false>(e0, transposeWithDegree(e0), PagerankOptions<double>());
  if (!emp.ranks.empty() || emp.iterations != 0) { printf("empty graph: MISMATCH\n"); ++fails; }
  printf(fails ? "FAILED\n" : "OK\n");
  return fails ? 1 : 0;
}
