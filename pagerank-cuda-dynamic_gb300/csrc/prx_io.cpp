// prx_io.cpp -- edge-list readers of the C ABI (host, OpenMP; no device work).
//
// The reference reads its graphs with getline + istringstream on the host:
// SNAP temporal text in consecutive pieces (readTemporalDo,
// inc/snap.hxx:41-52; main.cu:167 takes the first 90% of the lines and
// main.cu:83 each batch after it) and MatrixMarket coordinate files
// (readMtxHeader inc/mtx.hxx:39-54, readMtxDo inc/mtx.hxx:119-135).  Here a
// buffered reader splits lines with memchr and parses a block of up to 2^20
// lines in parallel; the result is the same edge sequence.  Ids in the files
// are 1-based and come out 0-based; the edge list then goes to
// prx_graph_create_from_edges, which sorts, merges and transposes it on the
// device.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>
#include <omp.h>
#include "pagerank_gb300.h"
#include "prx_reader.h"

namespace prx {
void set_error(const std::string& msg);
}

namespace prx_io {

void fill(prx_edge_reader* r) {
  if (r->beg > 0) {
    std::memmove(r->buf.data(), r->buf.data() + r->beg, r->end - r->beg);
    r->end -= r->beg;
    r->beg = 0;
  }
  if (r->end == r->buf.size()) r->buf.resize(r->buf.size() * 2);
  const size_t got = std::fread(r->buf.data() + r->end, 1, r->buf.size() - r->end, r->f);
  r->end += got;
  if (got == 0) r->eof = true;
}

}  // namespace prx_io

namespace {

using prx_io::fill;
bool read_line(prx_edge_reader* r, std::string& line);
bool parse_u64(const char*& p, const char* e, uint64_t& out);

}  // namespace

namespace prx_io {

int mtx_header(prx_edge_reader* r, uint64_t* order, bool* symmetric) {
  // comment lines start with '%', the banner with "%%"; the first other line
  // holds rows, cols and the entry count
  std::string line, h0, h1, h2, h3, h4;
  for (;;) {
    if (!read_line(r, line)) line.clear();
    if (line.rfind('%', 0) != 0) break;
    if (line.rfind("%%", 0) != 0) continue;
    std::istringstream ss(line);
    ss >> h0 >> h1 >> h2 >> h3 >> h4;
  }
  *order = 0;
  *symmetric = false;
  if (h1 != "matrix" || h2 != "coordinate") return PRX_OK;
  *symmetric = h4 == "symmetric" || h4 == "skew-symmetric";
  uint64_t rows = 0, cols = 0, size = 0;
  const char* p = line.data();
  const char* e = p + line.size();
  if (parse_u64(p, e, rows) && parse_u64(p, e, cols) && parse_u64(p, e, size)) *order = std::max(rows, cols);
  return PRX_OK;
}

}  // namespace prx_io

namespace {

constexpr size_t kBufBytes = 64u << 20;
constexpr size_t kBlockLines = 1u << 20;

int fail(int code, const std::string& msg) {
  prx::set_error(msg);
  return code;
}

// One line (without its '\n') as std::getline gives it; false at the end.
bool read_line(prx_edge_reader* r, std::string& line) {
  for (;;) {
    const char* b = r->buf.data() + r->beg;
    const char* nl = (const char*)std::memchr(b, '\n', r->end - r->beg);
    if (nl) {
      line.assign(b, (size_t)(nl - b));
      r->beg = (size_t)(nl - r->buf.data()) + 1;
      return true;
    }
    if (r->eof) {
      if (r->beg == r->end) return false;
      line.assign(b, r->end - r->beg);
      r->beg = r->end;
      return true;
    }
    fill(r);
  }
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f' || c == '\n'; }

// Unsigned decimal after optional whitespace and '+', like operator>> into an
// unsigned integer; false if there are no digits or the value overflows.
bool parse_u64(const char*& p, const char* e, uint64_t& out) {
  while (p < e && is_space(*p)) ++p;
  if (p < e && *p == '+') ++p;
  if (p >= e || *p < '0' || *p > '9') return false;
  uint64_t x = 0;
  for (; p < e && *p >= '0' && *p <= '9'; ++p) {
    const uint64_t d = (uint64_t)(*p - '0');
    if (x > (UINT64_MAX - d) / 10) return false;
    x = x * 10 + d;
  }
  out = x;
  return true;
}

struct Span {
  size_t b, e, next;  // line bytes [b, e); the line after starts at next
};

// Read up to `size` lines of "u v ..." (1-based ids in 1..rows) into U, V
// (0-based; (v, u) after (u, v) when symmetric).  A line without two
// unsigned integers is consumed and ends the read.  *lines: lines consumed.
int read_edges(prx_edge_reader* r, uint64_t rows, uint64_t size, bool symmetric, std::vector<uint32_t>& U,
               std::vector<uint32_t>& V, uint64_t* lines) {
  uint64_t done = 0;
  std::vector<Span> spans;
  std::vector<uint64_t> pu, pv;
  std::vector<unsigned char> ok;
  while (done < size) {
    const char* b = r->buf.data() + r->beg;
    if (!std::memchr(b, '\n', r->end - r->beg) && !r->eof) {
      fill(r);
      continue;
    }
    // complete lines now in the buffer (and the unterminated last one at EOF)
    spans.clear();
    size_t p = r->beg;
    while (done + spans.size() < size && spans.size() < kBlockLines) {
      const char* q = (const char*)std::memchr(r->buf.data() + p, '\n', r->end - p);
      if (q) {
        const size_t e = (size_t)(q - r->buf.data());
        spans.push_back({p, e, e + 1});
        p = e + 1;
      } else if (r->eof && p < r->end) {
        spans.push_back({p, r->end, r->end});
        p = r->end;
      } else {
        break;
      }
    }
    if (spans.empty()) break;  // end of the file
    const int64_t cnt = (int64_t)spans.size();
    pu.resize(cnt);
    pv.resize(cnt);
    ok.resize(cnt);
    const char* base = r->buf.data();
#pragma omp parallel for schedule(static, 4096)
    for (int64_t i = 0; i < cnt; ++i) {
      const char* s = base + spans[i].b;
      const char* e = base + spans[i].e;
      ok[i] = parse_u64(s, e, pu[i]) && parse_u64(s, e, pv[i]);
    }
    int64_t stop = cnt;  // first line that failed to parse
    for (int64_t i = 0; i < cnt; ++i)
      if (!ok[i]) {
        stop = i;
        break;
      }
    int64_t bad = -1;  // first id outside 1..rows
    for (int64_t i = 0; i < stop && bad < 0; ++i)
      if (pu[i] < 1 || pu[i] > rows || pv[i] < 1 || pv[i] > rows) bad = i;
    if (bad >= 0) {
      char msg[160];
      std::snprintf(msg, sizeof msg, "edge reader: line %llu: vertex id outside 1..%llu",
                    (unsigned long long)(done + bad + 1), (unsigned long long)rows);
      return fail(PRX_EINVAL, msg);
    }
    const size_t at = U.size(), per = symmetric ? 2 : 1;
    U.resize(at + per * stop);
    V.resize(at + per * stop);
#pragma omp parallel for schedule(static, 4096)
    for (int64_t i = 0; i < stop; ++i) {
      const uint32_t u = (uint32_t)(pu[i] - 1), v = (uint32_t)(pv[i] - 1);
      U[at + per * i] = u;
      V[at + per * i] = v;
      if (symmetric) {
        U[at + per * i + 1] = v;
        V[at + per * i + 1] = u;
      }
    }
    if (stop < cnt) {
      r->beg = spans[stop].next;
      done += stop + 1;
      break;
    }
    r->beg = p;
    done += cnt;
  }
  *lines = done;
  return PRX_OK;
}

int hand_out(const std::vector<uint32_t>& U, const std::vector<uint32_t>& V, uint32_t** u, uint32_t** v,
             uint64_t* count) {
  const size_t m = U.size();
  *u = (uint32_t*)std::malloc(sizeof(uint32_t) * (m ? m : 1));
  *v = (uint32_t*)std::malloc(sizeof(uint32_t) * (m ? m : 1));
  if (!*u || !*v) {
    std::free(*u);
    std::free(*v);
    *u = *v = nullptr;
    return fail(PRX_ENOMEM, "edge reader: host allocation failed");
  }
  if (m) {
    std::memcpy(*u, U.data(), sizeof(uint32_t) * m);
    std::memcpy(*v, V.data(), sizeof(uint32_t) * m);
  }
  *count = m;
  return PRX_OK;
}

}  // namespace

extern "C" {

int prx_edge_reader_open(const char* path, prx_edge_reader** out) {
  if (!path || !out) return fail(PRX_EINVAL, "prx_edge_reader_open: NULL argument");
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(PRX_EINVAL, std::string("prx_edge_reader_open: cannot open ") + path);
  prx_edge_reader* r = new prx_edge_reader();
  r->f = f;
  r->buf.resize(kBufBytes);
  *out = r;
  return PRX_OK;
}

int prx_edge_reader_next(prx_edge_reader* r, uint32_t rows, uint64_t size, int symmetric, uint32_t** u,
                         uint32_t** v, uint64_t* count, uint64_t* lines) {
  if (!r || !u || !v || !count) return fail(PRX_EINVAL, "prx_edge_reader_next: NULL argument");
  *u = *v = nullptr;
  *count = 0;
  if (lines) *lines = 0;
  std::vector<uint32_t> U, V;
  uint64_t got = 0;
  if (rows != 0 && size != 0) {  // readTemporalDo reads nothing then (inc/snap.hxx:42)
    U.reserve((size_t)std::min<uint64_t>(size, 1u << 24) * (symmetric ? 2 : 1));
    V.reserve(U.capacity());
    const int rc = read_edges(r, rows, size, symmetric != 0, U, V, &got);
    if (rc != PRX_OK) return rc;
  }
  if (lines) *lines = got;
  return hand_out(U, V, u, v, count);
}

int prx_edge_reader_close(prx_edge_reader* r) {
  if (!r) return PRX_OK;
  if (r->f) std::fclose(r->f);
  delete r;
  return PRX_OK;
}

int prx_read_mtx(const char* path, uint32_t* n, uint32_t** u, uint32_t** v, uint64_t* count) {
  if (!path || !n || !u || !v || !count) return fail(PRX_EINVAL, "prx_read_mtx: NULL argument");
  *n = 0;
  *u = *v = nullptr;
  *count = 0;
  prx_edge_reader* r = nullptr;
  int rc = prx_edge_reader_open(path, &r);
  if (rc != PRX_OK) return rc;
  uint64_t order = 0;
  bool symmetric = false;
  rc = prx_io::mtx_header(r, &order, &symmetric);
  if (rc == PRX_OK && order >= 0xffffffffull) rc = fail(PRX_ERANGE, "prx_read_mtx: more than 2^32 - 2 vertices");
  std::vector<uint32_t> U, V;
  if (rc == PRX_OK && order > 0) {
    uint64_t got = 0;
    rc = read_edges(r, order, UINT64_MAX, symmetric, U, V, &got);
    if (rc == PRX_OK) *n = (uint32_t)order;
  }
  prx_edge_reader_close(r);
  if (rc != PRX_OK) return rc;
  return hand_out(U, V, u, v, count);
}

int prx_format_edges(const uint32_t* u, const uint32_t* v, uint64_t count, char** text, uint64_t* bytes) {
  // "u v\n" per edge, ids written 1-based (the readers' input format)
  if (!text || !bytes || (count && (!u || !v))) return fail(PRX_EINVAL, "prx_format_edges: NULL argument");
  *text = nullptr;
  *bytes = 0;
  auto digits = [](uint64_t x) {
    int d = 1;
    while (x >= 10) {
      x /= 10;
      ++d;
    }
    return d;
  };
  constexpr int64_t kBlock = 1 << 16;
  const int64_t blocks = (int64_t)((count + kBlock - 1) / kBlock);
  std::vector<uint64_t> off((size_t)blocks + 1, 0);
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < blocks; ++b) {
    uint64_t len = 0;
    for (uint64_t i = (uint64_t)b * kBlock; i < std::min<uint64_t>(count, (uint64_t)(b + 1) * kBlock); ++i)
      len += digits((uint64_t)u[i] + 1) + digits((uint64_t)v[i] + 1) + 2;
    off[b + 1] = len;
  }
  for (int64_t b = 0; b < blocks; ++b) off[b + 1] += off[b];
  char* out = (char*)std::malloc(off[blocks] ? off[blocks] : 1);
  if (!out) return fail(PRX_ENOMEM, "prx_format_edges: host allocation failed");
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < blocks; ++b) {
    char* p = out + off[b];
    for (uint64_t i = (uint64_t)b * kBlock; i < std::min<uint64_t>(count, (uint64_t)(b + 1) * kBlock); ++i) {
      for (int k = 0; k < 2; ++k) {
        uint64_t x = (uint64_t)(k ? v[i] : u[i]) + 1;
        const int d = digits(x);
        for (int q = d - 1; q >= 0; --q) {
          p[q] = (char)('0' + x % 10);
          x /= 10;
        }
        p += d;
        *p++ = k ? '\n' : ' ';
      }
    }
  }
  *text = out;
  *bytes = off[blocks];
  return PRX_OK;
}

int prx_format_glog(char* buf, size_t len, double deletions_fraction, double insertions_fraction, int batch_index,
                    int threads, const prx_result* r, double err, const char* technique) {
  // main.cu:56-59
  if (!r || !technique) return -PRX_EINVAL;
  return std::snprintf(buf, len,
                       "{-%.3e/+%.3e batchf, %03d batchi, %03d threads} -> {%09.1fms, %09.1fms init, %09.1fms mark, "
                       "%09.1fms comp, %03d iter, %.2e err} %s",
                       deletions_fraction, insertions_fraction, batch_index, threads, (double)r->time_ms,
                       (double)r->initialization_time_ms, (double)r->marking_time_ms,
                       (double)r->computation_time_ms, r->iterations, err, technique);
}

}  // extern "C"
