// ref_harness.cpp -- drives the reference's own CPU code to produce golden
// fixtures that pin the oracle.  TEST INFRASTRUCTURE ONLY.
//
// Built by oracle/Makefile (target `ref`) against the headers of
// puzzlef/pagerank-cuda-dynamic (inc/), only where those headers exist; the
// binary lands in oracle/_ref/ and is run by tests/golden/make_golden.py.
// Nothing in the product or in the GPU tests runs it.
//
// Input (stdin, text):
//   n m tol
//   m lines "u v"                  edges of x (self-loops included by caller)
//   nd, then nd lines "u v"        raw deletions (untidied)
//   ni, then ni lines "u v"        raw insertions (untidied)
// Output (stdout): records "name kind count" followed by count values
// (kind u = unsigned integers, f = doubles printed with %a).
#define BUILD 0
#define OPENMP 1
#include <cstdio>
#include <cstdint>
#include <vector>
#include <tuple>
#include "_main.hxx"
#include "Graph.hxx"
#include "csr.hxx"
#include "properties.hxx"
#include "duplicate.hxx"
#include "transpose.hxx"
#include "bfs.hxx"
#include "batch.hxx"
#include "pagerank.hxx"
#include "pagerankPrune.hxx"

using namespace std;
using K = uint32_t;

static void putU(const char* name, const vector<K>& a) {
  printf("%s u %zu\n", name, a.size());
  for (size_t i = 0; i < a.size(); ++i) printf("%u%c", a[i], (i + 1 == a.size()) ? '\n' : ' ');
  if (a.empty()) printf("\n");
}
static void putF(const char* name, const vector<double>& a) {
  printf("%s f %zu\n", name, a.size());
  for (size_t i = 0; i < a.size(); ++i) printf("%a%c", a[i], (i + 1 == a.size()) ? '\n' : ' ');
  if (a.empty()) printf("\n");
}
static void putI(const char* name, long v) { printf("%s u 1\n%ld\n", name, v); }

template <class G>
static void putCsr(const char* off, const char* edg, const G& x) {
  vector<K> ks = vertexKeys(x), o, e;
  csrCreateOffsetsW(o, x, ks);
  csrCreateEdgeKeysW(e, x, ks);
  putU(off, o);
  putU(edg, e);
}

template <class H>
static void putDat(const char* name, const H& xt) {
  vector<K> ks = vertexKeys(xt), d;
  csrCreateVertexValuesW(d, xt, ks);
  putU(name, d);
}

static void putEdges(const char* us, const char* vs, const vector<tuple<K, K>>& b) {
  vector<K> a, c;
  for (auto& [u, v] : b) { a.push_back(u); c.push_back(v); }
  putU(us, a);
  putU(vs, c);
}

int main() {
  size_t n, m;
  double tol;
  if (scanf("%zu %zu %lf", &n, &m, &tol) != 3) return 2;
  DiGraph<K> x;
  for (K u = 0; u < n; ++u) x.addVertex(u);
  for (size_t i = 0; i < m; ++i) {
    K u, v;
    if (scanf("%u %u", &u, &v) != 2) return 2;
    x.addEdge(u, v);
  }
  x.update();
  vector<tuple<K, K>> deletions, insertions;
  size_t nd, ni;
  if (scanf("%zu", &nd) != 1) return 2;
  for (size_t i = 0; i < nd; ++i) { K u, v; if (scanf("%u %u", &u, &v) != 2) return 2; deletions.push_back({u, v}); }
  if (scanf("%zu", &ni) != 1) return 2;
  for (size_t i = 0; i < ni; ++i) { K u, v; if (scanf("%u %u", &u, &v) != 2) return 2; insertions.push_back({u, v}); }

  auto xt = transposeWithDegreeOmp(x);
  putCsr("x_off", "x_edg", x);
  putCsr("xt_off", "xt_edg", xt);
  putDat("xt_dat", xt);
  PagerankOptions<double> o(1, tol);
  auto sx = pagerankStaticOmp(xt, o);
  putF("static_x_ranks", sx.ranks);
  putI("static_x_iters", sx.iterations);

  auto y = duplicate(x);
  tidyBatchUpdateU(deletions, insertions, y);
  applyBatchUpdateOmpU(y, deletions, insertions);
  auto yt = transposeWithDegreeOmp(y);
  putEdges("del_u", "del_v", deletions);
  putEdges("ins_u", "ins_v", insertions);
  putCsr("y_off", "y_edg", y);
  putCsr("yt_off", "yt_edg", yt);
  putDat("yt_dat", yt);

  vector<char> df(max(x.span(), y.span())), dt(max(x.span(), y.span()));
  pagerankAffectedFrontierW(df, x, y, deletions, insertions);
  pagerankAffectedTraversalW(dt, x, y, deletions, insertions);
  vector<K> dfu(df.begin(), df.end()), dtu(dt.begin(), dt.end());
  putU("df_flags", dfu);
  putU("dt_flags", dtu);

  auto sy = pagerankStaticOmp(yt, o);
  putF("static_y_ranks", sy.ranks);
  putI("static_y_iters", sy.iterations);
  auto ny = pagerankNaiveDynamic<false>(yt, &sx.ranks, o);
  putF("nd_y_ranks", ny.ranks);
  putI("nd_y_iters", ny.iterations);
  // Converged answer on y, the reference's error yardstick (main.cu:88).
  auto zy = pagerankStaticOmp(yt, PagerankOptions<double>(1, 1e-100));
  putF("exact_y_ranks", zy.ranks);
  return 0;
}
