// prx_parse.cu -- edge-list text parsed on the device.
//
// The reference reads "u v ..." lines with getline + istringstream on the host
// (readTemporalDo, inc/snap.hxx:41-52; readMtxDo, inc/mtx.hxx:119-135).  Here
// the bytes go to the device in chunks and are parsed there:
//   1. k_nl_count: newlines per 64 KB block (16-byte loads, byte compares);
//   2. an exclusive scan of the block counts gives each block its first line;
//   3. k_parse_lines: each block lists the starts of the lines after its
//      newlines in shared memory, and its threads parse consecutive lines of
//      the list together (line 0 by the first thread).  Ids are 1-based in
//      the text and stored 0-based; the first line that does not start with
//      two unsigned integers and the first id outside 1..rows are found with
//      atomicMin, so the result is the same line sequence the host reader
//      gives: every line before the first bad one, at most `size` of them.
// The edges stay on the device and feed prx_graph_create_from_edges_device's
// sort / merge / transpose directly.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include "prx_ctx.h"
#include "prx_reader.h"

namespace prx {

constexpr int kParseThreads = 256;
constexpr int kParseBytes = 256;                               // bytes per thread
constexpr uint64_t kParseBlock = (uint64_t)kParseThreads * kParseBytes;  // 64 KB per block

__device__ __forceinline__ uint32_t nl_in_word(uint32_t w) { return __popc(__vcmpeq4(w, 0x0A0A0A0Au)) >> 3; }

// newlines in this thread's 256 bytes (the buffer is zero-padded to whole blocks)
__device__ __forceinline__ uint32_t nl_in_segment(const uint4* seg) {
  uint32_t c = 0;
#pragma unroll
  for (int q = 0; q < kParseBytes / 16; ++q) {
    const uint4 x = seg[q];
    c += nl_in_word(x.x) + nl_in_word(x.y) + nl_in_word(x.z) + nl_in_word(x.w);
  }
  return c;
}

__global__ void __launch_bounds__(kParseThreads) k_nl_count(const uint4* __restrict__ text, uint32_t* __restrict__ block_nl) {
  __shared__ uint32_t ws[kParseThreads / 32];
  const uint32_t c = nl_in_segment(text + ((uint64_t)blockIdx.x * kParseBlock + threadIdx.x * kParseBytes) / 16);
  uint32_t x = c;
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int k = 0; k < kParseThreads / 32; ++k) s += ws[k];
    block_nl[blockIdx.x] = s;
  }
}

__device__ __forceinline__ bool line_space(uint8_t c) {
  return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f';
}

// operator>> into an unsigned integer, within one line: blanks, an optional
// '+', digits; false without digits or on overflow.
__device__ __forceinline__ bool dev_parse_u64(const uint8_t* __restrict__ t, uint64_t& p, uint64_t end,
                                              unsigned long long& out) {
  while (p < end && line_space(t[p])) ++p;
  if (p < end && t[p] == '+') ++p;
  if (p >= end || t[p] < '0' || t[p] > '9') return false;
  unsigned long long x = 0;
  for (; p < end && t[p] >= '0' && t[p] <= '9'; ++p) {
    const unsigned long long d = t[p] - '0';
    if (x > (~0ull - d) / 10) return false;
    x = x * 10 + d;
  }
  out = x;
  return true;
}

struct ParseArgs {
  const uint8_t* text;
  uint64_t bytes;              // valid bytes of the chunk
  const uint32_t* nl_base;     // newlines before each block (exclusive scan)
  uint64_t lines;              // lines in the chunk (complete ones, plus the last one at EOF)
  uint64_t limit;              // lines wanted (<= lines)
  uint64_t rows;
  int symmetric;
  uint32_t* u;                 // outputs, indexed by line (x2 when symmetric)
  uint32_t* v;
  unsigned long long* fail;    // first line that does not parse
  unsigned long long* bad;     // first line with an id outside 1..rows
};

__device__ void parse_line(const ParseArgs& a, uint64_t k, uint64_t s) {
  // the line runs from s to the next newline or the chunk end
  uint64_t end = s;
  while (end < a.bytes && a.text[end] != '\n') ++end;
  uint64_t p = s;
  unsigned long long x = 0, y = 0;
  if (!(dev_parse_u64(a.text, p, end, x) && dev_parse_u64(a.text, p, end, y))) {
    atomicMin(a.fail, (unsigned long long)k);
    return;
  }
  if (x < 1 || x > a.rows || y < 1 || y > a.rows) {
    atomicMin(a.bad, (unsigned long long)k);
    return;
  }
  const uint32_t uu = (uint32_t)(x - 1), vv = (uint32_t)(y - 1);
  if (a.symmetric) {
    a.u[2 * k] = uu;
    a.v[2 * k] = vv;
    a.u[2 * k + 1] = vv;
    a.v[2 * k + 1] = uu;
  } else {
    a.u[k] = uu;
    a.v[k] = vv;
  }
}

// Parse pass.  A thread parsing the lines after its own newlines would leave
// the lanes of a warp in different lines at different times (each lane owns
// a different number of newlines per word), so the lines would be parsed one
// lane at a time.  Instead the block first lists the starts of the lines
// that follow its newlines in shared memory (kLineCap at a time), then the
// threads take consecutive lines from the list together.
constexpr int kLineCap = 8192;

__global__ void __launch_bounds__(kParseThreads) k_parse_lines(ParseArgs a) {
  __shared__ uint32_t ws[kParseThreads / 32];
  __shared__ uint32_t starts[kLineCap];  // block-relative start of each listed line
  const uint64_t block0 = (uint64_t)blockIdx.x * kParseBlock;
  const uint32_t off0 = threadIdx.x * kParseBytes;  // this thread's bytes, block-relative
  const uint4* seg = reinterpret_cast<const uint4*>(a.text + block0 + off0);
  const uint32_t c = nl_in_segment(seg);
  // newlines of this block before this thread's bytes, and in the whole block
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = c;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  uint32_t ex = x - c, total = 0;
  for (int k = 0; k < kParseThreads / 32; ++k) {
    if (k < (int)w) ex += ws[k];
    total += ws[k];
  }
  const uint64_t j0 = a.nl_base[blockIdx.x];  // newlines before this block
  if (block0 == 0 && threadIdx.x == 0 && a.limit > 0) parse_line(a, 0, 0);
  for (uint32_t lo = 0; lo < total; lo += kLineCap) {
    const uint32_t hi = lo + kLineCap;
    if (c && ex < hi && ex + c > lo) {
      uint32_t q = ex;  // block-local number of the next newline of this thread
      for (int v16 = 0; v16 < kParseBytes / 16 && q < hi; ++v16) {
        const uint4 vv = seg[v16];
        const uint32_t wd[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          uint32_t m = __vcmpeq4(wd[e], 0x0A0A0A0Au);
          while (m) {
            const int bit = __ffs(m) - 1;  // lowest byte first: the text's order
            m &= ~(0xFFu << bit);
            if (q >= lo && q < hi) starts[q - lo] = off0 + v16 * 16 + e * 4 + (bit >> 3) + 1;
            ++q;
          }
        }
      }
    }
    __syncthreads();
    const uint32_t cnt = (total < hi ? total : hi) - lo;
    for (uint32_t i = threadIdx.x; i < cnt; i += kParseThreads) {
      const uint64_t k = j0 + lo + i + 1;  // the line after block newline lo + i
      if (k < a.limit && k < a.lines) parse_line(a, k, block0 + starts[i]);
    }
    __syncthreads();
  }
}

// Position of newline number target (0-based) in the chunk -> *out.
__global__ void __launch_bounds__(kParseThreads) k_find_newline(const uint8_t* __restrict__ text,
                                                                const uint32_t* __restrict__ nl_base,
                                                                uint32_t blocks, uint64_t target,
                                                                unsigned long long* __restrict__ out) {
  __shared__ uint32_t ws[kParseThreads / 32];
  const uint64_t lo = nl_base[blockIdx.x];
  const uint64_t hi = blockIdx.x + 1 < blocks ? nl_base[blockIdx.x + 1] : ~0ull;
  if (target < lo || target >= hi) return;
  const uint64_t seg0 = (uint64_t)blockIdx.x * kParseBlock + (uint64_t)threadIdx.x * kParseBytes;
  const uint4* seg = reinterpret_cast<const uint4*>(text + seg0);
  const uint32_t c = nl_in_segment(seg);
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = c;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  uint64_t j = lo + x - c;
  for (uint32_t k = 0; k < w; ++k) j += ws[k];
  if (target < j || target >= j + c) return;
  for (int q = 0; q < kParseBytes; ++q) {
    if (text[seg0 + q] != '\n') continue;
    if (j == target) {
      *out = seg0 + q;
      return;
    }
    ++j;
  }
}

}  // namespace prx

namespace {

using namespace prx;

// Device edge list under construction (grows by doubling).
struct DevEdges {
  uint32_t* u = nullptr;
  uint32_t* v = nullptr;
  uint64_t n = 0, cap = 0;
  cudaError_t reserve(uint64_t want, cudaStream_t s) {
    if (want <= cap) return cudaSuccess;
    uint64_t nc = std::max<uint64_t>(want, cap * 2);
    uint32_t *nu = nullptr, *nv = nullptr;
    cudaError_t e = graph_alloc(&nu, 4 * nc, s);
    if (e == cudaSuccess) e = graph_alloc(&nv, 4 * nc, s);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(nu, u, 4 * n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(nv, v, 4 * n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      graph_free({nu, nv});
      return e;
    }
    graph_free({u, v});
    u = nu;
    v = nv;
    cap = nc;
    return cudaSuccess;
  }
  void release() {
    graph_free({u, v});
    u = v = nullptr;
    n = cap = 0;
  }
};

// Parse scratch reused across chunks.
struct ParseBufs {
  uint8_t* text = nullptr;
  uint64_t text_cap = 0;
  uint32_t* nl = nullptr;
  uint64_t nl_cap = 0;
  unsigned long long* word = nullptr;  // [0] fail, [1] bad, [2] newline position
  ~ParseBufs() { graph_free({text, nl, word}); }
};

int parse_fail(cudaError_t e) {
  set_error(std::string("edge text parse: ") + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
}

// Parse up to `want` lines of chunk[0 .. bytes) (host memory) onto the end of
// E.  at_eof: the chunk ends the input (its last line may lack a newline);
// otherwise the bytes after the last newline are left unread.  *lines_used
// and *bytes_used: what was consumed (the line that ended the read
// included); *stopped: a line failed to parse.
int parse_chunk(prx_context* c, ParseBufs& B, const char* chunk, uint64_t bytes, bool at_eof, uint64_t rows,
                uint64_t want, bool symmetric, DevEdges& E, uint64_t* lines_used, uint64_t* bytes_used,
                bool* stopped) {
  cudaStream_t s = c->stream;
  *lines_used = *bytes_used = 0;
  *stopped = false;
  if (bytes == 0 || want == 0) return PRX_OK;
  // below 4 GB a chunk has fewer than 2^32 newlines, so the 32-bit scan holds
  if (bytes >= (1ull << 32)) FAIL(PRX_ERANGE, "edge text parse: chunk of 4 GB or more");
  const uint64_t blocks64 = (bytes + kParseBlock - 1) / kParseBlock;
  const uint32_t blocks = (uint32_t)blocks64;
  const uint64_t padded = blocks64 * kParseBlock;
  cudaError_t e = cudaSuccess;
  if (B.text_cap < padded) {
    graph_free({B.text});
    B.text = nullptr;
    B.text_cap = 0;
    e = graph_alloc(&B.text, padded, s);
    if (e != cudaSuccess) return parse_fail(e);
    B.text_cap = padded;
  }
  if (B.nl_cap < blocks64 + 1) {
    graph_free({B.nl});
    B.nl = nullptr;
    B.nl_cap = 0;
    e = graph_alloc(&B.nl, 4 * (blocks64 + 1), s);
    if (e != cudaSuccess) return parse_fail(e);
    B.nl_cap = blocks64 + 1;
  }
  if (!B.word) {
    e = graph_alloc(&B.word, 3 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return parse_fail(e);
  }
  e = cudaMemcpyAsync(B.text, chunk, bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && padded > bytes) e = cudaMemsetAsync(B.text + bytes, 0, padded - bytes, s);
  if (e != cudaSuccess) return parse_fail(e);
  k_nl_count<<<blocks, kParseThreads, 0, s>>>(reinterpret_cast<const uint4*>(B.text), B.nl);
  e = cudaMemsetAsync(B.nl + blocks, 0, 4, s);
  if (e == cudaSuccess) e = exclusive_scan_u32(B.nl, blocks + 1, s);
  uint32_t nl_total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&nl_total, B.nl + blocks, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return parse_fail(e);
  const bool unterminated = at_eof && chunk[bytes - 1] != '\n';
  const uint64_t lines = (uint64_t)nl_total + (unterminated ? 1 : 0);
  const uint64_t limit = std::min(lines, want);
  if (limit == 0) return PRX_OK;
  const uint64_t per = symmetric ? 2 : 1;
  e = E.reserve(E.n + per * limit, s);
  if (e != cudaSuccess) return parse_fail(e);
  const unsigned long long init[3] = {~0ull, ~0ull, ~0ull};
  e = cudaMemcpyAsync(B.word, init, sizeof init, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return parse_fail(e);
  ParseArgs a;
  a.text = B.text;
  a.bytes = bytes;
  a.nl_base = B.nl;
  a.lines = lines;
  a.limit = limit;
  a.rows = rows;
  a.symmetric = symmetric ? 1 : 0;
  a.u = E.u + E.n;
  a.v = E.v + E.n;
  a.fail = B.word;
  a.bad = B.word + 1;
  k_parse_lines<<<blocks, kParseThreads, 0, s>>>(a);
  unsigned long long w[2] = {0, 0};
  e = cudaMemcpyAsync(w, B.word, sizeof w, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return parse_fail(e);
  const uint64_t good = std::min<uint64_t>(w[0], limit);  // lines before the first that fails
  if (w[1] < good) {
    char msg[160];
    std::snprintf(msg, sizeof msg, "edge text parse: line %llu of the piece: vertex id outside 1..%llu",
                  (unsigned long long)w[1] + 1, (unsigned long long)rows);
    FAIL(PRX_EINVAL, msg);
  }
  E.n += per * good;
  *stopped = w[0] < limit;
  const uint64_t consumed = good + (*stopped ? 1 : 0);
  *lines_used = consumed;
  if (consumed == lines && unterminated) {
    *bytes_used = bytes;
  } else {
    // the consumed lines end at newline number consumed - 1
    const unsigned long long none = ~0ull;
    e = cudaMemcpyAsync(B.word + 2, &none, sizeof none, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      k_find_newline<<<blocks, kParseThreads, 0, s>>>(B.text, B.nl, blocks, consumed - 1, B.word + 2);
    unsigned long long pos = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&pos, B.word + 2, sizeof pos, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return parse_fail(e);
    if (pos >= bytes) FAIL(PRX_ECUDA, "edge text parse: newline position not found");
    *bytes_used = pos + 1;
  }
  return PRX_OK;
}

// Parse up to `size` lines from text[0 .. bytes) in device chunks of at most
// `chunk_max` bytes.
int parse_text(prx_context* c, const char* text, uint64_t bytes, bool at_eof, uint64_t rows, uint64_t size,
               bool symmetric, DevEdges& E, uint64_t* lines_out, uint64_t* bytes_out) {
  constexpr uint64_t kChunk = 1ull << 30;
  ParseBufs B;
  uint64_t off = 0, lines = 0;
  uint64_t chunk_max = kChunk;
  while (lines < size && off < bytes) {
    const uint64_t len = std::min(chunk_max, bytes - off);
    const bool last = off + len == bytes;
    uint64_t lu = 0, bu = 0;
    bool stopped = false;
    const int st = parse_chunk(c, B, text + off, len, last && at_eof, rows, size - lines, symmetric, E, &lu, &bu,
                               &stopped);
    if (st) return st;
    lines += lu;
    off += bu;
    if (stopped) break;
    if (bu == 0) {
      if (last) break;                       // no complete line left
      chunk_max *= 2;                        // one line longer than a chunk
      if (chunk_max >= (1ull << 32)) FAIL(PRX_ERANGE, "edge text parse: line too long");
    }
  }
  *lines_out = lines;
  *bytes_out = off;
  return PRX_OK;
}

int finish_graph(prx_context* c, uint32_t n, DevEdges& E, int self_loops, prx_graph** out) {
  const int st = prx_graph_create_from_edges_device(c, n, E.u, E.v, E.n, self_loops, out);
  E.release();
  return st;
}

}  // namespace

extern "C" {

int prx_graph_create_from_text(prx_context* c, const char* text, uint64_t bytes, uint32_t rows, uint64_t size,
                               int symmetric, int self_loops, prx_graph** out, uint64_t* lines, uint64_t* used) {
  if (!c || !out || (bytes && !text)) FAIL(PRX_EINVAL, "prx_graph_create_from_text: NULL argument");
  *out = nullptr;
  if (lines) *lines = 0;
  if (used) *used = 0;
  TRY_CUDA_ST(cudaSetDevice(c->device));
  DevEdges E;
  uint64_t l = 0, b = 0;
  if (rows != 0 && size != 0) {  // readTemporalDo reads nothing then (inc/snap.hxx:42)
    const int st = parse_text(c, text, bytes, true, rows, size, symmetric != 0, E, &l, &b);
    if (st) {
      E.release();
      return st;
    }
  }
  const int st = finish_graph(c, rows, E, self_loops, out);
  if (st == PRX_OK) {
    if (lines) *lines = l;
    if (used) *used = b;
  }
  return st;
}

int prx_edge_reader_next_graph(prx_edge_reader* r, prx_context* c, uint32_t rows, uint64_t size, int symmetric,
                               int self_loops, prx_graph** out, uint64_t* lines) {
  if (!r || !c || !out) FAIL(PRX_EINVAL, "prx_edge_reader_next_graph: NULL argument");
  *out = nullptr;
  if (lines) *lines = 0;
  TRY_CUDA_ST(cudaSetDevice(c->device));
  DevEdges E;
  ParseBufs B;
  uint64_t done = 0;
  if (rows != 0 && size != 0) {
    while (done < size) {
      if (r->beg == r->end || (!r->eof && !std::memchr(r->buf.data() + r->beg, '\n', r->end - r->beg))) {
        if (r->eof) break;
        prx_io::fill(r);
        continue;
      }
      uint64_t lu = 0, bu = 0;
      bool stopped = false;
      const int st = parse_chunk(c, B, r->buf.data() + r->beg, r->end - r->beg, r->eof, rows, size - done,
                                 symmetric != 0, E, &lu, &bu, &stopped);
      if (st) {
        E.release();
        return st;
      }
      done += lu;
      r->beg += bu;
      if (stopped) break;
      if (done < size && !r->eof) prx_io::fill(r);
      else if (r->eof && r->beg == r->end) break;
    }
  }
  const int st = finish_graph(c, rows, E, self_loops, out);
  if (st == PRX_OK && lines) *lines = done;
  return st;
}

int prx_graph_create_from_mtx(prx_context* c, const char* path, int self_loops, prx_graph** out, uint32_t* n_out) {
  if (!c || !path || !out) FAIL(PRX_EINVAL, "prx_graph_create_from_mtx: NULL argument");
  *out = nullptr;
  if (n_out) *n_out = 0;
  prx_edge_reader* r = nullptr;
  int st = prx_edge_reader_open(path, &r);
  if (st) return st;
  uint64_t order = 0;
  bool symmetric = false;
  st = prx_io::mtx_header(r, &order, &symmetric);
  if (st == PRX_OK && order >= 0xffffffffull) {
    set_error("prx_graph_create_from_mtx: more than 2^32 - 2 vertices");
    st = PRX_ERANGE;
  }
  if (st == PRX_OK)
    st = prx_edge_reader_next_graph(r, c, (uint32_t)order, order ? ~0ull : 0, symmetric ? 1 : 0, self_loops, out,
                                    nullptr);
  prx_edge_reader_close(r);
  if (st == PRX_OK && n_out) *n_out = (uint32_t)order;
  return st;
}

}  // extern "C"
