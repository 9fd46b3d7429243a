// prx_graph.cu -- device-side graph preparation.
//
// build_classes(): the reference splits vertices into in-degree <= 64 and
// > 64 with two CUB scans, two scatters and a blocking copy of the split
// point (pagerankPartitionVerticesCuW, inc/pagerankCuda.hxx:625-638), rebuilt
// inside every timed solve (:812-813).  Here one stable 3-way partition
// (LOW / MID / HIGH, ids ascending within each class) is built once per graph
// version with three kernels of our own and reused by every solve on it.
#include <algorithm>
#include <mutex>
#include <vector>
#include "prx_device.cuh"

namespace prx {

namespace {
constexpr int kMaxDevices = 64;
cudaMemPool_t g_pool[kMaxDevices] = {};
std::mutex g_pool_mu;

cudaError_t pool_of(int dev, cudaMemPool_t* out) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(pool);
      return e;
    }
    g_pool[dev] = pool;
  }
  *out = g_pool[dev];
  return cudaSuccess;
}
}  // namespace

cudaError_t graph_alloc(void** p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  cudaMemPool_t pool = nullptr;
  if (e == cudaSuccess) e = pool_of(dev, &pool);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync(p, bytes ? bytes : 1, pool, s);
  return e;
}

void graph_free(std::initializer_list<void*> ps) {
  bool any = false;
  for (void* p : ps) any = any || p;
  if (!any) return;
  cudaDeviceSynchronize();
  for (void* p : ps)
    if (p) cudaFreeAsync(p, cudaStreamLegacy);
  // the blocks are free before the next allocation on any stream looks
  cudaStreamSynchronize(cudaStreamLegacy);
}

cudaError_t graph_pool_trim(int dev) {
  cudaMemPool_t pool = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (dev < 0 || dev >= kMaxDevices || !g_pool[dev]) return cudaSuccess;
    pool = g_pool[dev];
  }
  return cudaMemPoolTrimTo(pool, 0);
}

cudaError_t graph_pool_stats(int dev, uint64_t out[4]) {
  for (int k = 0; k < 4; ++k) out[k] = 0;
  cudaMemPool_t pool = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (dev < 0 || dev >= kMaxDevices || !g_pool[dev]) return cudaSuccess;
    pool = g_pool[dev];
  }
  const cudaMemPoolAttr attrs[4] = {cudaMemPoolAttrReservedMemCurrent, cudaMemPoolAttrReservedMemHigh,
                                    cudaMemPoolAttrUsedMemCurrent, cudaMemPoolAttrUsedMemHigh};
  for (int k = 0; k < 4; ++k) {
    const cudaError_t e = cudaMemPoolGetAttribute(pool, attrs[k], &out[k]);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

constexpr uint32_t kTileV = 2048;            // vertices per tile (256 threads x 8)
constexpr int kFieldBits = 21;               // per-class count within a tile, packed into a u64
constexpr unsigned long long kFieldMask = (1ull << kFieldBits) - 1;

__device__ __forceinline__ unsigned long long cls_code(const uint32_t* __restrict__ xtoff, uint32_t shift, uint32_t v,
                                                     uint32_t mid_max) {
  return 1ull << (kFieldBits * in_class(xtoff, shift, v, mid_max));
}

// Inclusive scan over a 256-thread block; *total receives the block sum.
__device__ __forceinline__ unsigned long long block_scan_incl(unsigned long long x, unsigned long long* total) {
  __shared__ unsigned long long wsum[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  unsigned long long pre = 0, tot = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    if (i < w) pre += wsum[i];
    tot += wsum[i];
  }
  *total = tot;
  __syncthreads();
  return x + pre;
}

// Per-tile class counts, class-major: cnt[c * ntiles + tile].
__global__ void __launch_bounds__(256) k_cls_count(const uint32_t* __restrict__ xtoff, uint32_t shift, uint32_t n, uint32_t mid_max,
                                                   uint32_t ntiles, uint32_t* __restrict__ cnt) {
  const uint32_t v0 = blockIdx.x * kTileV + threadIdx.x * 8;
  unsigned long long x = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if (v0 + k < n) x += cls_code(xtoff, shift, v0 + k, mid_max);
  unsigned long long tot;
  block_scan_incl(x, &tot);
  if (threadIdx.x == 0)
    for (int c = 0; c < NCLS; ++c) cnt[c * ntiles + blockIdx.x] = (uint32_t)((tot >> (kFieldBits * c)) & kFieldMask);
}

// One block of 1024 threads: exclusive scan of cnt[0 .. len) in place (the
// class-major layout makes the result the global start of each (class, tile)),
// plus the class boundaries bounds[0..3].
__global__ void __launch_bounds__(1024) k_cls_scan(uint32_t* cnt, uint32_t ntiles, uint32_t* bounds) {
  __shared__ uint32_t sh[1024];
  const uint32_t len = NCLS * ntiles;
  const uint32_t t = threadIdx.x;
  const uint32_t per = (len + 1023) / 1024;
  const uint32_t b = min(len, t * per), e = min(len, b + per);
  uint32_t local = 0;
  for (uint32_t i = b; i < e; ++i) local += cnt[i];
  sh[t] = local;
  __syncthreads();
  for (uint32_t o = 1; o < 1024; o <<= 1) {
    const uint32_t y = t >= o ? sh[t - o] : 0;
    __syncthreads();
    sh[t] += y;
    __syncthreads();
  }
  uint32_t run = t ? sh[t - 1] : 0;
  for (uint32_t i = b; i < e; ++i) {
    const uint32_t x = cnt[i];
    cnt[i] = run;
    if (i % ntiles == 0) bounds[i / ntiles] = run;
    run += x;
  }
  if (t == 1023) bounds[NCLS] = sh[1023];
}

__global__ void __launch_bounds__(256) k_cls_scatter(const uint32_t* __restrict__ xtoff, uint32_t shift, uint32_t n, uint32_t mid_max,
                                                     uint32_t ntiles, const uint32_t* __restrict__ start,
                                                     uint32_t* __restrict__ out) {
  const uint32_t v0 = blockIdx.x * kTileV + threadIdx.x * 8;
  int cls[8];
  unsigned long long x = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    cls[k] = v0 + k < n ? in_class(xtoff, shift, v0 + k, mid_max) : -1;
    if (cls[k] >= 0) x += 1ull << (kFieldBits * cls[k]);
  }
  unsigned long long tot;
  unsigned long long pos = block_scan_incl(x, &tot) - x;  // exclusive, packed per class
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (cls[k] < 0) continue;
    const int c = cls[k];
    const uint32_t local = (uint32_t)((pos >> (kFieldBits * c)) & kFieldMask);
    out[start[c * ntiles + blockIdx.x] + local] = v0 + k;
    pos += 1ull << (kFieldBits * c);
  }
}

// In-edges per class (statistics for the roofline): one u64 atomic per block
// and class.
__global__ void __launch_bounds__(256) k_cls_edges(const uint32_t* __restrict__ xtoff, uint32_t shift, uint32_t n, uint32_t mid_max,
                                                   unsigned long long* __restrict__ out) {
  __shared__ unsigned long long acc[NCLS];
  if (threadIdx.x < NCLS) acc[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long mine[NCLS] = {0, 0, 0};
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    mine[in_class(xtoff, shift, v, mid_max)] += row_len(xtoff, shift, v);
  for (int c = 0; c < NCLS; ++c)
    if (mine[c]) atomicAdd(&acc[c], mine[c]);
  __syncthreads();
  if (threadIdx.x < NCLS && acc[threadIdx.x]) atomicAdd(&out[threadIdx.x], acc[threadIdx.x]);
}

// RN(1/d) for every out-degree below kRcpTable, formed by the same divisions
// as k_reciprocals (FP64 division is many FP64 instructions on this part, and
// 50M vertices share a few thousand degrees).  Filled before each use on the
// stream that reads it.
constexpr uint32_t kRcpTable = 1u << 16;
__device__ double g_rcp_table[kRcpTable];
__device__ float g_rcp32_table[kRcpTable];

__global__ void k_rcp_table() {
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < kRcpTable; d += gridDim.x * blockDim.x) {
    g_rcp_table[d] = 1.0 / (double)d;
    g_rcp32_table[d] = 1.0f / (float)d;
  }
}

__global__ void k_reciprocals(const uint32_t* __restrict__ deg, uint32_t n, double* __restrict__ rcp,
                              float* __restrict__ rcp32) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const uint32_t d = deg[v];
    rcp[v] = d < kRcpTable ? g_rcp_table[d] : 1.0 / (double)d;
    rcp32[v] = d < kRcpTable ? g_rcp32_table[d] : 1.0f / (float)d;
  }
}

// Self-test of div_count against the IEEE division: d in [1, dmax] and
// `per` dividends per d spread over 2^-40 .. 2^2 (mantissas from a hash).
__global__ void k_selftest_div(uint32_t dmax, uint32_t per, unsigned long long* bad) {
  unsigned long long mine = 0;
  const uint64_t total = (uint64_t)dmax * per;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t d = (uint32_t)(i / per) + 1;
    uint64_t z = i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const int ex = 1023 - 40 + (int)((z >> 52) % 43);
    const double a = __longlong_as_double((long long)(((uint64_t)ex << 52) | (z & 0xFFFFFFFFFFFFFull)));
    const double y = 1.0 / (double)d;
    if (dbits(div_count(a, d, y)) != dbits(a / (double)d)) ++mine;
    if (dbits(u32_to_f64(d)) != dbits((double)d) || (i == 0 && dbits(u32_to_f64(0)) != 0)) ++mine;
    // the tolerance comparisons of a relative change |m - b| / max(m, b)
    // around their tie band: b = m -+ c*m*(1 + t 2^-50) for t in [-2^8, 2^8)
    // (+-1024 ulps about c*m), c = 1e-6 * (1 + small), either argument order;
    // every 64th case with b negated (the division path)
    const double m = a;
    const double c = 1e-6 * (1.0 + (double)(z & 0xffff) * 0x1p-20);
    const double t = (double)((int)((z >> 16) & 0x1ff) - 256);
    const double xx = c * m * (1.0 + t * 0x1p-50);
    double b = ((z >> 25) & 1) ? m - xx : m + xx;
    if (((z >> 27) & 63) == 0) b = -b;
    const RelChange rc = ((z >> 26) & 1) ? rel_change(m, b) : rel_change(b, m);
    const double q = fabs(m - b) / fmax(m, b);
    if (quot_le(rc, c) != (q <= c) || quot_gt(rc, c) != (q > c)) ++mine;
  }
  if (mine) atomicAdd(bad, mine);
}

cudaError_t selftest_division(uint32_t dmax, uint32_t per, unsigned long long* bad_host, int sms, cudaStream_t s) {
  unsigned long long* bad = nullptr;
  cudaError_t e = graph_alloc(&bad, sizeof(*bad), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(*bad), s);
  if (e == cudaSuccess) {
    k_selftest_div<<<sms * 8, 256, 0, s>>>(dmax, per, bad);
    e = cudaMemcpyAsync(bad_host, bad, sizeof(*bad), cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  graph_free({bad});
  return e;
}

// Bitmap of the LOW class (warp per 32 ids).
__global__ void __launch_bounds__(256) k_low_bitmap(const uint32_t* __restrict__ xtoff, uint32_t shift, uint32_t n,
                                                    uint32_t* __restrict__ bm) {
  const uint32_t words = (n + 31) >> 5;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (w << 5) | (threadIdx.x & 31u);
    const bool low = v < n && row_len(xtoff, shift, v) <= kLowMax;
    const unsigned b = __ballot_sync(0xffffffffu, low);
    if ((threadIdx.x & 31u) == 0) bm[w] = b;
  }
}

// Per (chunk, vertex) in-edge counts of the LOW class, chunk-major, with a
// zero at the end of every chunk row (so one exclusive scan gives offsets).
__global__ void k_chunk_count(const uint32_t* __restrict__ xtoff, const uint32_t* __restrict__ xtedg,
                              const uint32_t* __restrict__ low_bm, uint32_t n, uint32_t width, int K,
                              uint32_t* __restrict__ cnt) {
  const size_t row = (size_t)n + 1;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x) {
    const bool low = v < n && ((low_bm[v >> 5] >> (v & 31u)) & 1u);
    uint32_t j = low ? xtoff[v] : 0, e = low ? xtoff[v + 1] : 0;
    for (int k = 0; k < K; ++k) {
      const uint64_t hi = (uint64_t)(k + 1) * width;
      const uint32_t b = j;
      while (j < e && xtedg[j] < hi) ++j;
      cnt[k * row + v] = j - b;
    }
  }
}


__global__ void k_chunk_scatter(const uint32_t* __restrict__ xtoff, const uint32_t* __restrict__ xtedg,
                                const uint32_t* __restrict__ low_bm, uint32_t n, uint32_t width, int K,
                                const uint32_t* __restrict__ off, uint32_t* __restrict__ edg,
                                const uint32_t* __restrict__ hot_idx, uint32_t hot_words) {
  const size_t row = (size_t)n + 1;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    if (!((low_bm[v >> 5] >> (v & 31u)) & 1u)) continue;
    uint32_t j = xtoff[v];
    const uint32_t e = xtoff[v + 1];
    for (int k = 0; k < K; ++k) {
      const uint64_t hi = (uint64_t)(k + 1) * width;
      uint32_t pos = off[k * row + v];
      while (j < e && xtedg[j] < hi) edg[pos++] = layout_id(hot_idx, hot_words, xtedg[j++]);
    }
  }
}

// Scatter for K <= kScatterK chunks, coalesced: a warp takes 32 consecutive
// rows (lane i: row v0+i) and walks the edges of each run of consecutive LOW
// rows among them -- one contiguous range of at most 32 x 64 edges -- 32
// edges at a time.  Each edge finds its row by a binary search over the
// lanes' row starts (the last row starting at or before it: empty rows are
// skipped that way) and its destination -- chunk k's piece of the row, which
// is a consecutive run since rows are sorted by source -- by shuffles from
// that row's lane.  The edges of rows of other classes (a hub row can hold
// millions) are never read.
constexpr int kScatterK = 8;
__global__ void __launch_bounds__(256) k_chunk_scatter_w(const uint32_t* __restrict__ xtoff,
                                                         const uint32_t* __restrict__ xtedg,
                                                         const uint32_t* __restrict__ low_bm, uint32_t n,
                                                         uint32_t width, int K, const uint32_t* __restrict__ off,
                                                         uint32_t* __restrict__ edg,
                                                         const uint32_t* __restrict__ hot_idx, uint32_t hot_words,
                                                         uint32_t g0 = 0,
                                                         uint32_t g1 = 0xffffffffu, uint64_t cap = ~0ull) {
  const size_t row = (size_t)n + 1;
  const uint32_t lane = lane_id();
  const uint32_t groups = min((n + 31) >> 5, g1);
  for (uint32_t gi = g0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); gi < groups;
       gi += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (gi << 5) + lane;
    const uint32_t s = xtoff[min(v, n)];
    const uint32_t end = xtoff[min((gi << 5) + 32u, n)];
    const bool low = v < n && ((low_bm[v >> 5] >> (v & 31u)) & 1u);
    uint32_t dst[kScatterK], rs[kScatterK];
    uint32_t run = 0;
#pragma unroll
    for (int k = 0; k < kScatterK; ++k) {
      dst[k] = 0;
      rs[k] = run;
      if (low && k < K) {
        dst[k] = off[k * row + v];
        run += off[k * row + v + 1] - dst[k];
      }
    }
    // runs of LOW rows [ra, rb): lanes past the group's end count as not LOW
    const unsigned lowm = __ballot_sync(0xffffffffu, low);
    for (unsigned rest = lowm; rest;) {
      const uint32_t ra = __ffs(rest) - 1;
      const unsigned above = ~rest & ~((1u << ra) - 1u);   // not LOW, at or after ra
      const uint32_t rb = above ? (uint32_t)(__ffs(above) - 1) : 32u;
      rest &= rb < 32 ? ~((1u << rb) - 1u) : 0u;
      const uint32_t rs0 = __shfl_sync(0xffffffffu, s, ra);
      const uint32_t run_end = rb < 32 ? __shfl_sync(0xffffffffu, s, rb) : end;
    // four 32-edge windows per step, their loads issued together
    for (uint32_t base = rs0; base < run_end; base += 128) {
      uint32_t uu[4];
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const uint32_t j = base + 32u * w + lane;
        uu[w] = j < run_end ? __ldg(xtedg + j) : 0u;
      }
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const uint32_t j = base + 32u * w + lane;
        uint32_t r = 0;
#pragma unroll
        for (int step = 16; step; step >>= 1) {
          const uint32_t cand = r + step;
          if (__shfl_sync(0xffffffffu, s, cand) <= j) r = cand;
        }
        const bool rlow = __shfl_sync(0xffffffffu, (int)low, r) != 0;
        const uint32_t sr = __shfl_sync(0xffffffffu, s, r);
        const bool act = j < run_end && rlow;
        const uint32_t u = uu[w];
        uint32_t k = 0;  // u's chunk: the chunk bounds at or below u (no division)
#pragma unroll
        for (int kk = 1; kk < kScatterK; ++kk)
          k += (kk < K && (uint64_t)u >= (uint64_t)kk * width) ? 1u : 0u;
        uint32_t d = 0, rr = 0;
#pragma unroll
        for (int kk = 0; kk < kScatterK; ++kk) {
          if (kk >= K) break;
          const uint32_t dk = __shfl_sync(0xffffffffu, dst[kk], r);
          const uint32_t rk = __shfl_sync(0xffffffffu, rs[kk], r);
          if (k == (uint32_t)kk) {
            d = dk;
            rr = rk;
          }
        }
        const uint64_t at = (uint64_t)d + (j - sr - rr);
        if (act && at < cap) edg[at] = layout_id(hot_idx, hot_words, u);
      }
    }
    }
  }
}

static void free_layout(ChunkLayout& l) {
  graph_free({l.off, l.edg});
  for (auto p : l.seg_off) graph_free({p});
  for (auto p : l.seg_edg) graph_free({p});
  l = ChunkLayout();
}

void free_chunks(GraphDev& g) {
  for (auto& l : g.lay) free_layout(l);
}

// The chunk layout of one CSR of `rows` rows (offsets off[0 .. rows], edges
// edg, LOW bitmap from its first row): counts, scan, scatter.
cudaError_t build_layout_into(const uint32_t* off, const uint32_t* edg, const uint32_t* low_bm, uint32_t rows,
                              uint32_t width, int K, const uint32_t* hot_idx, uint32_t hot_words, uint32_t* lay_off,
                              uint32_t* lay_edg, uint32_t* scan_ws, int sms, cudaStream_t s) {
  const size_t len = (size_t)K * ((size_t)rows + 1);
  if (len > 0xffffffffull) return cudaErrorInvalidValue;
  const int grid = sms * 8;
  k_chunk_count<<<grid, 256, 0, s>>>(off, edg, low_bm, rows, width, K, lay_off);
  cudaError_t e = exclusive_scan_u32_ws(lay_off, (uint32_t)len, scan_ws, s);
  if (e == cudaSuccess) {
    if (K <= kScatterK)
      k_chunk_scatter_w<<<grid, 256, 0, s>>>(off, edg, low_bm, rows, width, K, lay_off, lay_edg, hot_idx, hot_words);
    else
      k_chunk_scatter<<<grid, 256, 0, s>>>(off, edg, low_bm, rows, width, K, lay_off, lay_edg, hot_idx, hot_words);
    e = cudaGetLastError();
  }
  return e;
}

static cudaError_t build_layout(const uint32_t* off, const uint32_t* edg, const uint32_t* low_bm, uint32_t rows,
                                uint64_t low_edges, uint32_t width, int K, int sms, cudaStream_t s,
                                uint32_t** lay_off, uint32_t** lay_edg, const uint32_t* hot_idx,
                                uint32_t hot_words) {
  const size_t len = (size_t)K * ((size_t)rows + 1);
  if (len > 0xffffffffull) return cudaErrorInvalidValue;
  uint32_t* ws = nullptr;
  cudaError_t e = graph_alloc(lay_off, sizeof(uint32_t) * len, s);
  if (e == cudaSuccess) e = graph_alloc(lay_edg, sizeof(uint32_t) * edge_slots(low_edges), s);
  if (e == cudaSuccess) e = graph_alloc(&ws, sizeof(uint32_t) * scan_ws_words((uint32_t)len), s);
  if (e == cudaSuccess)
    e = build_layout_into(off, edg, low_bm, rows, width, K, hot_idx, hot_words, *lay_off, *lay_edg, ws, sms, s);
  if (ws) cudaFreeAsync(ws, s);
  return e;
}

static uint64_t g_layout_clock = 0;  // stamps of the layout slots (least recently used is rebuilt)

// ---- the default layout, built while the in-edges upload ---------------------
// Counts of rows [r0, r1) per chunk into cnt (chunk-major, K x (n+1)), and
// the piece's total per chunk into tot[k] (one atomic per warp and chunk).
__global__ void k_chunk_count_range(const uint32_t* __restrict__ xtoff, const uint32_t* __restrict__ xtedg,
                                    const uint32_t* __restrict__ low_bm, uint32_t n, uint32_t r0, uint32_t r1,
                                    uint32_t width, int K, uint32_t* __restrict__ cnt, uint32_t* __restrict__ tot) {
  const size_t row = (size_t)n + 1;
  const uint32_t span = r1 - r0;
  const uint32_t stride = gridDim.x * blockDim.x;
  // every lane runs the same trip count (the warp sums below are collective)
  for (uint32_t base = blockIdx.x * blockDim.x; base < span; base += stride) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = r0 + i;
    const bool low = i < span && ((low_bm[v >> 5] >> (v & 31u)) & 1u);
    uint32_t j = low ? xtoff[v] : 0, e = low ? xtoff[v + 1] : 0;
    for (int k = 0; k < K; ++k) {
      const uint64_t hi = (uint64_t)(k + 1) * width;
      const uint32_t b = j;
      while (j < e && xtedg[j] < hi) ++j;
      if (i < span) cnt[k * row + v] = j - b;
      uint32_t c = j - b;
      for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
      if (lane_id() == 0 && c) atomicAdd(tot + k, c);
    }
  }
}

// Out-edges of the sources of each chunk: a bound on the chunk's in-edges
// in the layout, known before the in-edges themselves.
__global__ void k_chunk_bounds(const uint32_t* __restrict__ xtdat, uint32_t n, uint32_t width, int K,
                               unsigned long long* __restrict__ bound) {
  for (int k = 0; k < K; ++k) {
    const uint64_t lo = (uint64_t)k * width, hi = lo + width < n ? lo + width : n;
    unsigned long long x = 0;
    for (uint64_t u = lo + blockIdx.x * blockDim.x + threadIdx.x; u < hi; u += gridDim.x * blockDim.x) x += xtdat[u];
    block_sum_u64(x, bound + k);
  }
}

// After the piece's per-chunk exclusive scans: add the chunk's base in the
// edge array (the bounds of the chunks before it) and the totals of the
// pieces before this one (tot holds P x K totals), and write the offset of
// row r1 (the next piece's first row, or the end of the chunk).
__global__ void k_chunk_carry(uint32_t* __restrict__ off, uint32_t n, uint32_t r0, uint32_t r1, int K,
                              const uint32_t* __restrict__ tot, int p, const unsigned long long* __restrict__ bound) {
  const size_t row = (size_t)n + 1;
  for (int k = 0; k < K; ++k) {
    uint32_t carry = 0;
    for (int q = 0; q < k; ++q) carry += (uint32_t)bound[q];
    for (int q = 0; q < p; ++q) carry += tot[q * K + k];
    for (uint32_t v = r0 + blockIdx.x * blockDim.x + threadIdx.x; v < r1; v += gridDim.x * blockDim.x)
      off[k * row + v] += carry;
    if (blockIdx.x == 0 && threadIdx.x == 0) off[k * row + r1] = carry + tot[p * K + k];
  }
}

cudaError_t build_default_layout_pipelined(GraphDev& g, uint32_t width, bool hot, int pieces,
                                           const uint32_t* piece_rows, const cudaEvent_t* piece_ready, int sms,
                                           cudaStream_t s) {
  if (width == 0 || g.n == 0 || g.nseg > 1) return cudaSuccess;
  if (hot && !g.hot_n) hot = false;
  const uint32_t n = g.n;
  if (width >= n) {  // one chunk: a layout only to encode hot sources (the solve reads the CSR otherwise)
    if (g.cls_begin[1] == g.cls_begin[0] || !hot) return cudaSuccess;
    width = n;
  }
  const int K = (int)((n + (uint64_t)width - 1) / width);
  if (K > kScatterK) return cudaSuccess;  // left to the first solve
  const size_t len = (size_t)K * ((size_t)n + 1);
  if (len > 0xffffffffull) return cudaSuccess;
  ChunkLayout* l = &g.lay[0];
  for (auto& x : g.lay)
    if (x.width == 0 || (l->width != 0 && x.stamp < l->stamp)) l = &x;
  free_layout(*l);
  // chunk k's edges go to a region of its sources' out-edge count, placed
  // after the regions of chunks 0 .. k-1 (the regions add up to m)
  uint32_t* tot = nullptr;
  unsigned long long* bound = nullptr;
  cudaError_t e = graph_alloc(&l->off, sizeof(uint32_t) * len, s);
  if (e == cudaSuccess) e = graph_alloc(&l->edg, sizeof(uint32_t) * edge_slots(g.m), s);
  if (e == cudaSuccess) e = graph_alloc(&tot, sizeof(uint32_t) * (size_t)pieces * K, s);
  if (e == cudaSuccess) e = graph_alloc(&bound, sizeof(unsigned long long) * K, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(tot, 0, sizeof(uint32_t) * (size_t)pieces * K, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(bound, 0, sizeof(unsigned long long) * K, s);
  unsigned long long hb[kScatterK] = {};
  if (e == cudaSuccess) {
    k_chunk_bounds<<<sms * 4, 256, 0, s>>>(g.xtdat, n, width, K, bound);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(hb, bound, sizeof(unsigned long long) * K, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  uint64_t sum_bound = 0;
  for (int k = 0; k < K; ++k) sum_bound += hb[k];
  const uint64_t cap = edge_slots(g.m);
  if (e == cudaSuccess && sum_bound > g.m) {  // out-degrees inconsistent with m: leave it to the first solve
    cudaFreeAsync(tot, s);
    cudaFreeAsync(bound, s);
    free_layout(*l);
    return cudaSuccess;
  }
  const uint32_t* hot_idx = hot ? g.hot_idx : nullptr;
  for (int p = 0; p < pieces && e == cudaSuccess; ++p) {
    const uint32_t r0 = piece_rows[p], r1 = piece_rows[p + 1];
    e = cudaStreamWaitEvent(s, piece_ready[p], 0);
    if (e != cudaSuccess || r0 == r1) continue;
    k_chunk_count_range<<<sms * 8, 256, 0, s>>>(g.xtoff, g.xtedg, g.low_bm, n, r0, r1, width, K, l->off,
                                                tot + (size_t)p * K);
    for (int k = 0; k < K && e == cudaSuccess; ++k)
      e = exclusive_scan_u32(l->off + (size_t)k * (n + 1) + r0, r1 - r0, s);
    if (e != cudaSuccess) break;
    k_chunk_carry<<<sms * 4, 256, 0, s>>>(l->off, n, r0, r1, K, tot, p, bound);
    k_chunk_scatter_w<<<sms * 8, 256, 0, s>>>(g.xtoff, g.xtedg, g.low_bm, n, width, K, l->off, l->edg, hot_idx,
                                              (n + 31) >> 5, r0 >> 5, (r1 + 31) >> 5, cap);
    e = cudaGetLastError();
  }
  // every chunk must have stayed within its region (the out-degrees bound it)
  std::vector<uint32_t> ht((size_t)pieces * K);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ht.data(), tot, sizeof(uint32_t) * ht.size(), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (tot) cudaFreeAsync(tot, s);
  if (bound) cudaFreeAsync(bound, s);
  bool fits = true;
  for (int k = 0; k < K && e == cudaSuccess; ++k) {
    uint64_t t = 0;
    for (int p = 0; p < pieces; ++p) t += ht[(size_t)p * K + k];
    fits = fits && t <= hb[k];
  }
  if (e != cudaSuccess || !fits) {
    free_layout(*l);
    return e;
  }
  l->width = width;
  l->K = K;
  l->hot = hot;
  l->stamp = ++g_layout_clock;
  return cudaSuccess;
}

cudaError_t ensure_chunks(GraphDev& g, uint32_t width, int sms, cudaStream_t s, const ChunkLayout** out,
                          bool hot) {
  uint64_t& clock = g_layout_clock;
  *out = nullptr;
  if (width == 0 || g.n == 0) return cudaSuccess;
  if (hot && !g.hot_n) hot = false;
  if (width >= g.n) {  // one chunk: the row-major CSR is the layout, unless hot sources are encoded
    if (g.cls_begin[1] == g.cls_begin[0] || !hot) return cudaSuccess;
    width = g.n;
  }
  if (g.nseg > 1 && g.seg_shift < 5) return cudaSuccess;  // segments must start on a LOW-bitmap word
  for (auto& l : g.lay)
    if (l.width == width && l.hot == hot) {
      l.stamp = ++clock;
      *out = &l;
      return cudaSuccess;
    }
  // an empty slot, else the least recently used one (never one handed out
  // for the current solve: those were used last)
  ChunkLayout* pick = &g.lay[0];
  for (auto& l : g.lay)
    if (l.width == 0 || (pick->width != 0 && l.stamp < pick->stamp)) pick = &l;
  ChunkLayout& l = *pick;
  free_layout(l);
  const uint32_t* hot_idx = hot ? g.hot_idx : nullptr;
  const int K = (int)((g.n + (uint64_t)width - 1) / width);
  cudaError_t e = cudaSuccess;
  if (g.nseg <= 1) {
    e = build_layout(g.xtoff, g.xtedg, g.low_bm, g.n, g.cls_edges[LOW], width, K, sms, s, &l.off, &l.edg, hot_idx,
                     (g.n + 31) / 32);
  } else {
    // one layout per row segment: its rows' offsets are a plain CSR of the
    // segment's edges; sources keep their global ids, so the chunks are global
    for (uint32_t q = 0; q < g.nseg && e == cudaSuccess; ++q) {
      const uint64_t v0 = (uint64_t)q << g.seg_shift;
      const uint32_t rows = (uint32_t)(std::min<uint64_t>(g.n, v0 + (1ull << g.seg_shift)) - v0);
      const uint64_t seg_edges_bound =
          (q + 1 < g.nseg ? g.xtseg0[q + 1] : g.m) - g.xtseg0[q];  // every edge of the segment
      uint32_t *lo = nullptr, *le = nullptr;
      e = build_layout(g.xtoff + v0 + q, g.xtedg + g.xtpos[q], g.low_bm + (v0 >> 5), rows, seg_edges_bound, width,
                       K, sms, s, &lo, &le, hot_idx, (g.n + 31) / 32);
      l.seg_off.push_back(lo);
      l.seg_edg.push_back(le);
    }
  }
  if (e != cudaSuccess) {
    free_layout(l);
    return e;
  }
  l.width = width;
  l.K = K;
  l.hot = hot;
  l.stamp = ++clock;
  *out = &l;
  return cudaSuccess;
}

// ---- hot sources --------------------------------------------------------------
constexpr uint32_t kDegBins = 1u << 16;  // out-degree histogram (the last bin holds every larger degree)

// Out-degrees crowd into a few bins (every vertex of a grid has 5 to 7), so
// a warp adds each distinct degree once (__match_any_sync), and a block
// counts the degrees below kSmallBins in shared memory before adding them to
// the global bins.
constexpr uint32_t kSmallBins = 1024;
__global__ void __launch_bounds__(256) k_degree_hist(const uint32_t* __restrict__ xtdat, uint32_t n,
                                                     uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[kSmallBins];
  for (uint32_t i = threadIdx.x; i < kSmallBins; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  // the loop bound is the same for the whole block, so every warp stays converged for the match
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = base + threadIdx.x;
    const uint32_t d = v < n ? min(xtdat[v], kDegBins - 1) : 0xffffffffu;
    const unsigned same = __match_any_sync(0xffffffffu, d);
    if (d != 0xffffffffu && (uint32_t)(__ffs(same) - 1) == lane) {
      if (d < kSmallBins) atomicAdd(&sh[d], (uint32_t)__popc(same));
      else atomicAdd(&hist[d], (uint32_t)__popc(same));
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < kSmallBins; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// The hot bitmap (out-degree >= t) and its per-word counts (rank[words] = 0
// for the scan that turns them into counts before each word).
__global__ void k_hot_bitmap(const uint32_t* __restrict__ xtdat, uint32_t n, uint32_t t, uint32_t* __restrict__ bm,
                             uint32_t* __restrict__ rank) {
  const uint32_t words = (n + 31) >> 5;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w <= words; w += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = (w << 5) | lane_id();
    const unsigned b = __ballot_sync(0xffffffffu, v < n && xtdat[v] >= t);
    if (lane_id() == 0) {
      if (w < words) bm[w] = b;
      rank[w] = __popc(b);
    }
  }
}

// rank holds the counts before each word: the list of hot sources in id order
__global__ void k_hot_list(const uint32_t* __restrict__ bm, const uint32_t* __restrict__ rank, uint32_t words,
                           uint32_t* __restrict__ hot_list) {
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += gridDim.x * blockDim.x) {
    uint32_t i = rank[w];
    for (uint32_t b = bm[w]; b; b &= b - 1) hot_list[i++] = (w << 5) | (uint32_t)(__ffs(b) - 1);
  }
}

void free_hot(GraphDev& g) {
  graph_free({g.hot_idx, g.hot_list});
  g.hot_idx = g.hot_list = nullptr;
  g.hot_n = 0;
  g.hot_cap = 0;
  g.hot_built = false;
}

cudaError_t ensure_hot(GraphDev& g, uint32_t cap, int sms, cudaStream_t s) {
  if (g.hot_built && g.hot_cap == cap) return cudaSuccess;
  // layouts built with the old numbering must not be used again
  for (auto& l : g.lay)
    if (l.hot) free_layout(l);
  free_hot(g);
  g.hot_built = true;
  g.hot_cap = cap;
  const uint32_t n = g.n;
  if (cap == 0 || n == 0 || n >= kHotFlag) return cudaSuccess;
  uint32_t* hist = nullptr;
  cudaError_t e = graph_alloc(&hist, sizeof(uint32_t) * kDegBins, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(hist, 0, sizeof(uint32_t) * kDegBins, s);
  if (e == cudaSuccess) {
    k_degree_hist<<<sms * 4, 256, 0, s>>>(g.xtdat, n, hist);
    e = cudaGetLastError();
  }
  std::vector<uint32_t> h(kDegBins);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), hist, sizeof(uint32_t) * kDegBins, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(hist, s);  // stream-ordered: no device-wide wait (a graph upload may still run beside it)
  if (e != cudaSuccess) return e;
  // threshold t: the smallest degree with count(d >= t) <= cap, and at least
  // twice the average out-degree (a graph without skew gains nothing)
  uint64_t above = 0;
  uint32_t t = kDegBins;
  for (uint32_t b = kDegBins; b-- > 1;) {
    if (above + h[b] > cap) break;
    above += h[b];
    t = b;
  }
  const uint32_t floor_t = (uint32_t)std::min<uint64_t>(kDegBins - 1, (2 * g.m + n - 1) / n);
  t = std::max(t, std::max(floor_t, 2u));
  uint64_t count = 0;
  for (uint32_t b = t; b < kDegBins; ++b) count += h[b];
  if (count == 0 || t >= kDegBins) return cudaSuccess;
  const uint32_t words = (n + 31) / 32;
  e = graph_alloc(&g.hot_idx, sizeof(uint32_t) * (2 * (size_t)words + 1), s);
  if (e == cudaSuccess) e = graph_alloc(&g.hot_list, sizeof(uint32_t) * count, s);
  if (e == cudaSuccess) {
    k_hot_bitmap<<<sms * 8, 256, 0, s>>>(g.xtdat, n, t, g.hot_idx, g.hot_idx + words);
    e = exclusive_scan_u32(g.hot_idx + words, words + 1, s);
  }
  if (e == cudaSuccess) {
    k_hot_list<<<sms * 4, 256, 0, s>>>(g.hot_idx, g.hot_idx + words, words, g.hot_list);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    free_hot(g);
    return e;
  }
  g.hot_built = true;
  g.hot_cap = cap;
  g.hot_n = (uint32_t)count;
  return cudaSuccess;
}

cudaError_t build_classes(GraphDev& g, int sms, cudaStream_t s, bool keep_layouts) {
  const uint32_t n = g.n;
  if (!keep_layouts) {
    free_chunks(g);
    free_hot(g);
  }
  if (!g.low_bm) {
    cudaError_t e = graph_alloc(&g.low_bm, sizeof(uint32_t) * (((size_t)n + 31) / 32 + 1), s);
    if (e != cudaSuccess) return e;
  }
  if (!g.rcp) {
    cudaError_t e = graph_alloc(&g.rcp, sizeof(double) * (n ? n : 1), s);
    if (e != cudaSuccess) return e;
  }
  if (!g.rcp32) {
    cudaError_t e = graph_alloc(&g.rcp32, sizeof(float) * (n ? n : 1), s);
    if (e != cudaSuccess) return e;
  }
  launch_vertex_tables(g.xtoff, g.seg_shift, g.xtdat, n, g.low_bm, g.rcp, g.rcp32, sms, s);
  if (!g.cls_list) {
    cudaError_t e = graph_alloc(&g.cls_list, sizeof(uint32_t) * (n ? n : 1), s);
    if (e != cudaSuccess) return e;
  }
  return build_class_lists(g.xtoff, g.seg_shift, n, g.mid_max, g.cls_list, g.cls_begin, g.cls_edges, sms, s);
}

void launch_vertex_tables(const uint32_t* xtoff, uint32_t shift, const uint32_t* xtdat, uint32_t n, uint32_t* low_bm,
                          double* rcp, float* rcp32, int sms, cudaStream_t s) {
  if (!n) return;
  k_low_bitmap<<<sms * 4, 256, 0, s>>>(xtoff, shift, n, low_bm);
  k_rcp_table<<<kRcpTable / 256, 256, 0, s>>>();
  k_reciprocals<<<sms * 4, 256, 0, s>>>(xtdat, n, rcp, rcp32);
}

cudaError_t build_class_lists(const uint32_t* off, uint32_t shift, uint32_t n, uint32_t mid_max, uint32_t* list,
                              uint32_t begin[NCLS + 1], uint64_t edges_out[NCLS], int sms, cudaStream_t s) {
  if (n == 0) {
    for (int c = 0; c <= NCLS; ++c) begin[c] = 0;
    for (int c = 0; c < NCLS; ++c) edges_out[c] = 0;
    return cudaSuccess;
  }
  const uint32_t ntiles = (n + kTileV - 1) / kTileV;
  uint32_t* cnt = nullptr;
  // [class-major tile counts | 4 bounds | pad | 3 u64 edge sums]
  const size_t words = (size_t)NCLS * ntiles + NCLS + 1;
  const size_t bytes = ((words * sizeof(uint32_t) + 7) & ~(size_t)7) + NCLS * sizeof(unsigned long long);
  cudaError_t e = graph_alloc(&cnt, bytes, s);
  if (e != cudaSuccess) return e;
  uint32_t* bounds = cnt + (size_t)NCLS * ntiles;
  unsigned long long* edges = (unsigned long long*)((char*)cnt + ((words * sizeof(uint32_t) + 7) & ~(size_t)7));
  e = cudaMemsetAsync(edges, 0, NCLS * sizeof(unsigned long long), s);
  k_cls_count<<<ntiles, 256, 0, s>>>(off, shift, n, mid_max, ntiles, cnt);
  k_cls_scan<<<1, 1024, 0, s>>>(cnt, ntiles, bounds);
  k_cls_scatter<<<ntiles, 256, 0, s>>>(off, shift, n, mid_max, ntiles, cnt, list);
  k_cls_edges<<<sms * 4, 256, 0, s>>>(off, shift, n, mid_max, edges);
  uint32_t hb[NCLS + 1];
  unsigned long long he[NCLS];
  if (e == cudaSuccess) e = cudaMemcpyAsync(hb, bounds, sizeof(hb), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(he, edges, sizeof(he), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(cnt, s);
  if (e != cudaSuccess) return e;
  for (int c = 0; c <= NCLS; ++c) begin[c] = hb[c];
  for (int c = 0; c < NCLS; ++c) edges_out[c] = he[c];
  return cudaGetLastError();
}

}  // namespace prx

namespace prx {

// ---- exclusive scan of uint32 (in place), three passes ----------------------
__global__ void __launch_bounds__(256) k_scan_tile_sums(const uint32_t* __restrict__ in, uint32_t len,
                                                        uint32_t* __restrict__ sums) {
  const uint32_t i0 = blockIdx.x * kTileV + threadIdx.x * 8;
  unsigned long long x = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) x += i0 + k < len ? in[i0 + k] : 0u;
  unsigned long long tot;
  block_scan_incl(x, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = (uint32_t)tot;
}

__global__ void __launch_bounds__(1024) k_scan_single(uint32_t* a, uint32_t len) {
  __shared__ uint32_t sh[1024];
  const uint32_t t = threadIdx.x;
  const uint32_t per = (len + 1023) / 1024;
  const uint32_t b = min(len, t * per), e = min(len, b + per);
  uint32_t local = 0;
  for (uint32_t i = b; i < e; ++i) local += a[i];
  sh[t] = local;
  __syncthreads();
  for (uint32_t o = 1; o < 1024; o <<= 1) {
    const uint32_t y = t >= o ? sh[t - o] : 0;
    __syncthreads();
    sh[t] += y;
    __syncthreads();
  }
  uint32_t run = t ? sh[t - 1] : 0;
  for (uint32_t i = b; i < e; ++i) {
    const uint32_t x = a[i];
    a[i] = run;
    run += x;
  }
}

__global__ void __launch_bounds__(256) k_scan_apply(uint32_t* __restrict__ data, uint32_t len,
                                                    const uint32_t* __restrict__ tile_pre) {
  const uint32_t i0 = blockIdx.x * kTileV + threadIdx.x * 8;
  uint32_t v[8];
  unsigned long long x = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) { v[k] = i0 + k < len ? data[i0 + k] : 0u; x += v[k]; }
  unsigned long long tot;
  uint32_t run = tile_pre[blockIdx.x] + (uint32_t)(block_scan_incl(x, &tot) - x);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (i0 + k < len) data[i0 + k] = run;
    run += v[k];
  }
}

uint32_t scan_ws_words(uint32_t len) { return (len + kTileV - 1) / kTileV; }

cudaError_t exclusive_scan_u32_ws(uint32_t* data, uint32_t len, uint32_t* sums, cudaStream_t s) {
  if (len == 0) return cudaSuccess;
  const uint32_t ntiles = scan_ws_words(len);
  k_scan_tile_sums<<<ntiles, 256, 0, s>>>(data, len, sums);
  k_scan_single<<<1, 1024, 0, s>>>(sums, ntiles);
  k_scan_apply<<<ntiles, 256, 0, s>>>(data, len, sums);
  return cudaGetLastError();
}

cudaError_t exclusive_scan_u32(uint32_t* data, uint32_t len, cudaStream_t s) {
  if (len == 0) return cudaSuccess;
  uint32_t* sums = nullptr;
  cudaError_t e = graph_alloc(&sums, sizeof(uint32_t) * scan_ws_words(len), s);
  if (e != cudaSuccess) return e;
  e = exclusive_scan_u32_ws(data, len, sums, s);
  cudaFreeAsync(sums, s);
  return e;
}

}  // namespace prx
