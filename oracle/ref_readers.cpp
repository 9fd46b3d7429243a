// ref_readers.cpp -- drives the reference's own file readers and graph
// builder to produce golden fixtures for the edge-list readers and the
// device-side graph ingest.  TEST INFRASTRUCTURE ONLY.
//
// Built by oracle/Makefile (target `ref`) against the headers of
// puzzlef/pagerank-cuda-dynamic (inc/), only where those headers exist; the
// binary lands in oracle/_ref/ and is run by tests/golden/make_readers_golden.py.
//
//   ref_readers pieces <file> <rows> <size>...   readTemporalDo (inc/snap.hxx:41-52)
//                                                on one stream, once per size
//   ref_readers mtx <file>                       readMtxDo (inc/mtx.hxx:119-135)
//   ref_readers pipeline <file> <rows> <size> <batch_fraction> <batches>
//       the graph flow of main.cu:163-171 and :80-86: readTemporalOmpW of the
//       first 90% of the lines, addSelfLoopsOmp, transposeWithDegreeOmp; then
//       per batch: the next batch_fraction * size lines as insertions,
//       tidyBatchUpdateU and applyBatchUpdateOmpU on a copy of x,
//       transposeWithDegreeOmp, and the copy becomes x.
// Output (stdout): records "name u count" followed by count unsigned values.
// Vertex keys are printed as read (1-based); CSRs are over vertexKeys().
#define BUILD 0
#define OPENMP 1
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <string>
#include <tuple>
#include <vector>
#include "_main.hxx"
#include "Graph.hxx"
#include "csr.hxx"
#include "properties.hxx"
#include "duplicate.hxx"
#include "transpose.hxx"
#include "selfLoop.hxx"
#include "batch.hxx"
#include "snap.hxx"
#include "mtx.hxx"

using namespace std;
using K = uint32_t;

static void put(const char* name, const vector<size_t>& a) {
  printf("%s u %zu\n", name, a.size());
  for (size_t i = 0; i < a.size(); ++i) printf("%zu%c", a[i], (i + 1 == a.size()) ? '\n' : ' ');
  if (a.empty()) printf("\n");
}
template <class T>
static void putK(const char* name, const vector<T>& a) {
  vector<size_t> b(a.begin(), a.end());
  put(name, b);
}

template <class G>
static void putCsr(const string& pre, const G& x) {
  vector<K> ks = vertexKeys(x), o, e;
  csrCreateOffsetsW(o, x, ks);
  csrCreateEdgeKeysW(e, x, ks);
  putK((pre + "_off").c_str(), o);
  putK((pre + "_edg").c_str(), e);
  putK((pre + "_keys").c_str(), ks);
}
template <class H>
static void putDat(const string& name, const H& xt) {
  vector<K> ks = vertexKeys(xt), d;
  csrCreateVertexValuesW(d, xt, ks);
  putK(name.c_str(), d);
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const string mode = argv[1];
  const char* file = argv[2];
  if (mode == "pieces") {
    if (argc < 5) return 2;
    const size_t rows = strtoull(argv[3], nullptr, 10);
    ifstream s(file);
    for (int a = 4; a < argc; ++a) {
      vector<size_t> us, vs;
      auto fb = [&](auto u, auto v, auto w) { us.push_back(u); vs.push_back(v); };
      readTemporalDo(s, false, false, rows, strtoull(argv[a], nullptr, 10), fb);
      const string i = to_string(a - 4);
      put(("u" + i).c_str(), us);
      put(("v" + i).c_str(), vs);
    }
    return 0;
  }
  if (mode == "mtx") {
    vector<size_t> us, vs, hdr;
    auto fh = [&](auto symmetric, auto rows, auto cols, auto size) { hdr = {size_t(symmetric), rows, cols, size}; };
    auto fb = [&](auto u, auto v, auto w) { us.push_back(u); vs.push_back(v); };
    readMtxDo(file, false, fh, fb);
    put("header", hdr);
    put("u", us);
    put("v", vs);
    return 0;
  }
  if (mode == "pipeline") {
    if (argc < 7) return 2;
    const size_t rows = strtoull(argv[3], nullptr, 10);
    const size_t size = strtoull(argv[4], nullptr, 10);
    const double frac = strtod(argv[5], nullptr);
    const int batches = atoi(argv[6]);
    DiGraph<K> x;
    ifstream s(file);
    readTemporalOmpW(x, s, false, false, rows, size_t(0.90 * size));
    auto fl = [](auto u) { return true; };
    x = addSelfLoopsOmp(x, None(), fl);
    auto xt = transposeWithDegreeOmp(x);
    putCsr("x", x);
    putCsr("xt", xt);
    putDat("xt_dat", xt);
    vector<tuple<K, K>> deletions, insertions;
    for (int b = 0; b < batches; ++b) {
      auto y = duplicate(x);
      insertions.clear();
      auto fb = [&](auto u, auto v, auto w) { insertions.push_back({K(u), K(v)}); };
      readTemporalDo(s, false, false, rows, size_t(frac * size), fb);
      vector<size_t> ru, rv;
      for (auto& [u, v] : insertions) { ru.push_back(u); rv.push_back(v); }
      tidyBatchUpdateU(deletions, insertions, y);
      applyBatchUpdateOmpU(y, deletions, insertions);
      auto yt = transposeWithDegreeOmp(y);
      vector<size_t> iu, iv;
      for (auto& [u, v] : insertions) { iu.push_back(u); iv.push_back(v); }
      const string i = to_string(b);
      put(("raw_u" + i).c_str(), ru);
      put(("raw_v" + i).c_str(), rv);
      put(("ins_u" + i).c_str(), iu);
      put(("ins_v" + i).c_str(), iv);
      putCsr("y" + i, y);
      putCsr("yt" + i, yt);
      putDat("yt_dat" + i, yt);
      swap(x, y);  // the batches accumulate (main.cu:143)
    }
    return 0;
  }
  return 2;
}
