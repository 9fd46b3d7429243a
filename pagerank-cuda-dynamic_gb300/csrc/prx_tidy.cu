// prx_tidy.cu -- batch tidying and graph ingest on the device.
//
// Tidying: the reference's
// tidyBatchUpdateU (inc/batch.hxx:152-208), which runs on the host there:
// keep the deletions that exist in the graph and the insertions that do not,
// sort each list by (u, v) and drop duplicates.
//
//   1. existence: binary search of v in u's out-row (rows are ascending);
//   2. keys: a kept deletion is its out-CSR position (the positions order
//      like (u, v)); a kept insertion is u * 2^b + v with b = bits(n - 1);
//   3. an LSD radix sort of the keys, 8-bit digits, stable (our own: per-block
//      digit histograms, a digit-major scan, and a scatter that ranks equal
//      digits in element order with warp ballots);
//   4. unique: first occurrences kept (scan of flags), decoded back to (u, v).
//
// Ingest (prx_graph_create_from_edges): the reference builds its DiGraph from
// an edge list on the host (readTemporalOmpW, inc/snap.hxx:158-166; edges
// merged into sorted neighbour sets), adds a self-loop to every vertex
// (addSelfLoopsOmp, inc/selfLoop.hxx:60-66) and transposes it with the
// out-degrees (transposeWithDegreeOmp, inc/transpose.hxx:110-134).  Here:
// keys u * 2^b + v (plus v * 2^b + v for the self-loops), radix sort, unique,
// row starts from the sorted keys; the transpose the same from v * 2^b + u.
#include <algorithm>
#include <vector>
#include "prx_ctx.h"
#include "prx_device.cuh"
#include "prx_hash.h"

namespace prx {

constexpr int kRadix = 256;
constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;                      // elements per thread per tile
constexpr int kSortTile = kSortThreads * kSortItems;

// Position of edge (u, v) in the out-CSR, or UINT32_MAX.
__device__ __forceinline__ uint32_t edge_position(const uint32_t* __restrict__ xoff, const uint32_t* __restrict__ xedg,
                                                  uint32_t u, uint32_t v) {
  uint32_t lo = xoff[u], hi = xoff[u + 1];
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (xedg[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return (lo < xoff[u + 1] && xedg[lo] == v) ? lo : 0xffffffffu;
}

// Does the out-CSR with row segments (see GraphDev) hold edge (u, v)?
__device__ __forceinline__ bool seg_has_edge(const uint32_t* __restrict__ xoff, const uint32_t* __restrict__ xedg,
                                             const unsigned long long* __restrict__ base, uint32_t shift, uint32_t u,
                                             uint32_t v) {
  const uint64_t k = seg_index(u, shift);
  const uint32_t* row = seg_edges(xedg, base, shift, u);
  uint32_t lo = xoff[k], hi = xoff[k + 1];
  const uint32_t end = hi;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (row[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo < end && row[lo] == v;
}

// keep[i] = 1 for kept edges; key[i] = the edge's sort key: a deletion's
// out-CSR position with pos_keys (one row segment), else u * 2^vbits + v.
// Ids >= n (the device batch generator's empty slots) are never kept.
__global__ void k_tidy_keys(const uint32_t* __restrict__ xoff, const uint32_t* __restrict__ xedg,
                            const unsigned long long* __restrict__ base, uint32_t shift, uint32_t n,
                            const uint32_t* __restrict__ u, const uint32_t* __restrict__ v, uint32_t count,
                            int deletions, int pos_keys, int vbits, uint32_t* __restrict__ keep,
                            unsigned long long* __restrict__ key) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    if (u[i] >= n || v[i] >= n) {
      keep[i] = 0;
      key[i] = 0;
      continue;
    }
    const unsigned long long uv = ((unsigned long long)u[i] << vbits) | v[i];
    if (pos_keys) {
      const uint32_t p = edge_position(xoff, xedg, u[i], v[i]);
      keep[i] = (p != 0xffffffffu) == (deletions != 0);
      key[i] = deletions ? p : uv;
    } else {
      keep[i] = seg_has_edge(xoff, xedg, base, shift, u[i], v[i]) == (deletions != 0);
      key[i] = uv;
    }
  }
}

// out[pos[i]] = in[i] where flag[i] (pos: exclusive scan of flag).
__global__ void k_compact64(const unsigned long long* __restrict__ in, const uint32_t* __restrict__ flag,
                            const uint32_t* __restrict__ pos, uint32_t count, unsigned long long* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    if (flag[i]) out[pos[i]] = in[i];
}

// Lanes of the warp holding the same 8-bit digit d as this lane, among the
// lanes where act is set: eight ballots, one per digit bit.
__device__ __forceinline__ unsigned digit_peers(uint32_t d, bool act) {
  unsigned peers = __ballot_sync(0xffffffffu, act);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const bool bit = (d >> b) & 1u;
    const unsigned m = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? m : ~m;
  }
  return peers;
}

// Element order within a tile (both radix steps): warp w owns the
// kSortItems * 32 consecutive keys from tile0 + w * kSortItems * 32, read 32
// at a time (round r: tile0 + w * kSortItems * 32 + r * 32 + lane).

// Radix pass, step 1: per-tile digit counts, digit-major: hist[d * tiles + b].
// Each warp counts into its own shared histogram.
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const unsigned long long* __restrict__ key,
                                                             uint32_t count, int shift, uint32_t tiles,
                                                             uint32_t* __restrict__ hist) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ uint32_t cnt[kWarps][kRadix];
  const uint32_t t = threadIdx.x, w = t >> 5, lane = t & 31u;
  for (int k = 0; k < kWarps; ++k) cnt[k][t] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * kSortTile + w * (kSortItems * 32) + lane;
  unsigned long long k[kSortItems];  // all loads in flight before the first use
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const uint32_t i = base + r * 32;
    k[r] = i < count ? key[i] : 0ull;
  }
#pragma unroll
  for (int r = 0; r < kSortItems; ++r)
    if (base + r * 32 < count) atomicAdd(&cnt[w][(k[r] >> shift) & (kRadix - 1)], 1u);
  __syncthreads();
  uint32_t sum = 0;
  for (int q = 0; q < kWarps; ++q) sum += cnt[q][t];
  hist[t * tiles + blockIdx.x] = sum;
}

// ---- bulk copies (TMA, non-tensor) into shared memory, mbarrier-tracked ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Arrive on bar (its one expected arrival) announcing `bytes` of transfers,
// then copy `bytes` (a multiple of 16, both addresses 16-byte aligned) from
// global memory to shared memory; the copy completes the barrier's phase.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with this parity (try_wait itself suspends for
// a while per call); false after kWaitLimit calls.
constexpr uint32_t kWaitLimit = 1u << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Radix pass, step 2 (after the exclusive scan of hist, so start[d * tiles +
// b] is where tile b's keys of digit d go): stable scatter.  Persistent
// blocks take tiles b, b + grid, ...; each tile's 32 KB of keys comes in by a
// bulk copy (cp.async.bulk) into one of two shared-memory stages, the next
// tile's copy in flight while this one is ranked.  Each warp ranks its keys
// among equal digits round by round (earlier rounds: a running per-warp
// count; within the round: lanes below with the same digit, from
// digit_peers); the tile is laid out by digit in shared memory (digit start
// in the tile + keys of that digit in lower warps + rank) and written out in
// that order, so the keys of one digit leave as one contiguous, coalesced
// run.  in must hold 2 keys of slack past count (the last tile's copy is
// rounded up to 16 bytes).  A copy that does not arrive within the wait
// limit sets *err and ends the block.
constexpr uint32_t kScatterSmem = (3 * kSortTile) * 8 + (2 + kSortThreads / 32) * kRadix * 4 + 64;

__global__ void __launch_bounds__(kSortThreads, 2) k_radix_scatter(const unsigned long long* __restrict__ in,
                                                                   uint32_t count, int shift, uint32_t tiles,
                                                                   const uint32_t* __restrict__ start,
                                                                   unsigned long long* __restrict__ out,
                                                                   uint32_t* __restrict__ err) {
  constexpr int kWarps = kSortThreads / 32;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned long long* stage = reinterpret_cast<unsigned long long*>(smem);  // [2][kSortTile]
  unsigned long long* sk = stage + 2 * kSortTile;                          // the tile by digit
  uint32_t* gbase = reinterpret_cast<uint32_t*>(sk + kSortTile);           // global start of digit d's run
  uint32_t* tstart = gbase + kRadix;                                       // start of digit d in the tile
  uint32_t* wrun = tstart + kRadix;                                        // [kWarps][kRadix]
  uint32_t* wsum = wrun + kWarps * kRadix;                                 // [kWarps]
  uint64_t* bar = reinterpret_cast<uint64_t*>(wsum + 8);                   // [2]
  const uint32_t t = threadIdx.x, w = t >> 5, lane = t & 31u;
  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
  }
  __syncthreads();
  auto issue = [&](uint32_t tile, int buf) {  // thread 0
    const uint32_t first = tile * kSortTile;
    const uint32_t nk = min((uint32_t)kSortTile, count - first);
    bulk_load(stage + buf * kSortTile, in + first, (nk * 8u + 15u) & ~15u, &bar[buf]);
  };
  uint32_t parity = 0;  // bit k: the phase parity stage k waits for next
  uint32_t tile = blockIdx.x, it = 0;
  if (tile < tiles && t == 0) issue(tile, 0);
  const unsigned lt = (1u << lane) - 1u;
  for (; tile < tiles; tile += gridDim.x, ++it) {
    const int buf = it & 1;
    const uint32_t next = tile + gridDim.x;
    // the other stage was last read in the previous tile, before its final barrier
    if (next < tiles && t == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(next, buf ^ 1);
    }
    const bool ok = mbar_wait(&bar[buf], (parity >> buf) & 1u);
    parity ^= 1u << buf;
    if (!__syncthreads_and(ok)) {
      // give up on this block: record it and let the copy still in flight land
      if (t == 0) {
        atomicExch(err, 1u);
        if (next < tiles) mbar_wait(&bar[buf ^ 1], (parity >> (buf ^ 1)) & 1u);
      }
      __syncthreads();
      return;
    }
    const unsigned long long* keys = stage + buf * kSortTile;
    const uint32_t tile0 = tile * kSortTile;
    const size_t idx = (size_t)t * tiles + tile;
    const uint32_t s0 = start[idx];
    const uint32_t s1 = idx + 1 < (size_t)kRadix * tiles ? start[idx + 1] : count;
    const uint32_t c = s1 - s0;  // this tile's keys of digit t
    gbase[t] = s0;
    for (int k = 0; k < kWarps; ++k) wrun[k * kRadix + t] = 0;
    __syncthreads();
    const uint32_t lbase = w * (kSortItems * 32) + lane;  // this lane's first key in the tile
    uint32_t rank[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
      const uint32_t li = lbase + r * 32;
      const bool act = tile0 + li < count;
      const uint32_t d = (uint32_t)((keys[li] >> shift) & (kRadix - 1));
      const unsigned peers = digit_peers(d, act);
      const uint32_t below = __popc(peers & lt);
      rank[r] = act ? wrun[w * kRadix + d] + below : 0;
      __syncwarp();
      if (act && below == 0) wrun[w * kRadix + d] += __popc(peers);
      __syncwarp();
    }
    // exclusive block scan of c over the 256 digits -> tstart; per digit, the
    // keys in lower warps -> wrun
    uint32_t x = c;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t k = 0; k < w; ++k) before += wsum[k];
    tstart[t] = before + x - c;
    uint32_t acc = 0;
    for (int k = 0; k < kWarps; ++k) {
      const uint32_t v = wrun[k * kRadix + t];
      wrun[k * kRadix + t] = acc;
      acc += v;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
      const uint32_t li = lbase + r * 32;
      if (tile0 + li < count) {
        const unsigned long long key = keys[li];
        const uint32_t d = (uint32_t)((key >> shift) & (kRadix - 1));
        sk[tstart[d] + wrun[w * kRadix + d] + rank[r]] = key;
      }
    }
    __syncthreads();
    const uint32_t nt = count - tile0 < (uint32_t)kSortTile ? count - tile0 : (uint32_t)kSortTile;
    for (uint32_t j = t; j < nt; j += kSortThreads) {
      const unsigned long long key = sk[j];
      const uint32_t d = (uint32_t)((key >> shift) & (kRadix - 1));
      out[gbase[d] + (j - tstart[d])] = key;
    }
    __syncthreads();  // stage, sk and the counters are free for the next tile
  }
}

// flag[i] = 1 for the first of equal adjacent keys.
__global__ void k_first_flags(const unsigned long long* __restrict__ key, uint32_t count, uint32_t* __restrict__ flag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    flag[i] = (i == 0 || key[i] != key[i - 1]) ? 1u : 0u;
}

// Decode the unique keys at pos[i] (flag[i]) into (u, v); pos_keys: the
// keys are out-CSR positions.
__global__ void k_decode(const unsigned long long* __restrict__ key, const uint32_t* __restrict__ flag,
                         const uint32_t* __restrict__ pos, uint32_t count, int pos_keys, int vbits,
                         const uint32_t* __restrict__ xoff, uint32_t n, const uint32_t* __restrict__ xedg,
                         uint32_t* __restrict__ ou, uint32_t* __restrict__ ov) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    if (!flag[i]) continue;
    const unsigned long long k = key[i];
    uint32_t u, v;
    if (pos_keys) {  // out-CSR position: v from the edge, u the row holding it
      const uint32_t p = (uint32_t)k;
      v = xedg[p];
      uint32_t lo = 0, hi = n;  // last row whose start is <= p
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (xoff[mid] <= p) lo = mid;
        else hi = mid - 1;
      }
      u = lo;
    } else {
      u = (uint32_t)(k >> vbits);
      v = (uint32_t)(k & ((1ull << vbits) - 1));
    }
    ou[pos[i]] = u;
    ov[pos[i]] = v;
  }
}

// Stable LSD radix sort of keys[0 .. count) on their bits [lo, hi), 8 at a
// time (keys must be below 2^hi), ping-ponging with tmp; *out is the buffer
// holding the result.  hist: 256 * ceil(count / kSortTile) + 1 words.
size_t radix_hist_words(uint32_t count) { return (size_t)kRadix * ((count + kSortTile - 1) / kSortTile) + 1; }

cudaError_t radix_sort_u64(unsigned long long* keys, unsigned long long* tmp, uint32_t count, int lo, int hi,
                           uint32_t* hist, int sms, cudaStream_t s, unsigned long long** out) {
  const uint32_t tiles = (count + kSortTile - 1) / kSortTile;
  unsigned long long *src = keys, *dst = tmp;
  *out = src;
  if (count == 0 || lo >= hi) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_radix_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, kScatterSmem);
  uint32_t* err = nullptr;
  if (e == cudaSuccess) e = graph_alloc(&err, sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const uint32_t grid = std::min<uint32_t>(tiles, 2u * (uint32_t)sms);
  for (int shift = lo; shift < hi && e == cudaSuccess; shift += 8) {
    k_radix_hist<<<tiles, kSortThreads, 0, s>>>(src, count, shift, tiles, hist);
    e = exclusive_scan_u32(hist, (uint32_t)(kRadix * tiles), s);
    if (e != cudaSuccess) break;
    k_radix_scatter<<<grid, kSortThreads, kScatterSmem, s>>>(src, count, shift, tiles, hist, dst, err);
    std::swap(src, dst);
  }
  uint32_t herr = 0;
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(err, s);
  if (e == cudaSuccess && herr) e = cudaErrorLaunchTimeout;  // a bulk copy never arrived
  *out = src;
  return e;
}

static int grid_of(uint64_t work, int sms) {
  const uint64_t b = (work + 255) / 256;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(b, (uint64_t)sms * 16));
}

// Edge keys of the ingest: u * 2^b + v for the listed edges, then v * 2^b + v
// for every vertex when self-loops are added.  An id >= n sets *bad (its key
// is clamped into range; the caller fails the call).
__global__ void k_ingest_keys(const uint32_t* __restrict__ u, const uint32_t* __restrict__ v, uint32_t count,
                              uint32_t n, int self_loops, int vbits, unsigned long long* __restrict__ key,
                              uint32_t* __restrict__ bad) {
  const uint32_t total = count + (self_loops ? n : 0);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    if (i < count) {
      uint32_t a = u[i], b = v[i];
      if (a >= n || b >= n) {
        *bad = 1u;
        a = min(a, n - 1);
        b = min(b, n - 1);
      }
      key[i] = ((unsigned long long)a << vbits) | b;
    } else {
      key[i] = ((unsigned long long)(i - count) << vbits) | (i - count);
    }
  }
}

// Unique sorted keys: low halves to edg, and the swapped keys (transpose).
__global__ void k_ingest_split(const unsigned long long* __restrict__ key, const uint32_t* __restrict__ flag,
                               const uint32_t* __restrict__ pos, uint32_t count, int vbits, int make_swapped,
                               unsigned long long* __restrict__ uniq, unsigned long long* __restrict__ swapped) {
  const unsigned long long mask = (1ull << vbits) - 1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    if (!flag[i]) continue;
    const unsigned long long k = key[i];
    uniq[pos[i]] = k;
    if (make_swapped) swapped[pos[i]] = ((k & mask) << vbits) | (k >> vbits);
  }
}

// Row starts of unique sorted keys: off[w] = number of keys whose high part
// (the row) is below w, by binary search (rows without keys need no
// special case, however long the run of them).
__global__ void k_ingest_offsets(const unsigned long long* __restrict__ key, uint32_t count, int vbits, uint32_t n,
                                 uint32_t* __restrict__ off) {
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w <= n; w += gridDim.x * blockDim.x) {
    const unsigned long long first = (unsigned long long)w << vbits;  // smallest key of row w
    uint32_t lo = 0, hi = count;
    while (lo < hi) {
      const uint32_t mid = lo + ((hi - lo) >> 1);
      if (key[mid] < first) lo = mid + 1;
      else hi = mid;
    }
    off[w] = lo;
  }
}

// Column ids of unique sorted keys: edg[i] = low part of key[i].
__global__ void k_ingest_columns(const unsigned long long* __restrict__ key, uint32_t count, int vbits,
                                 uint32_t* __restrict__ edg) {
  const unsigned long long mask = (1ull << vbits) - 1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    edg[i] = (uint32_t)(key[i] & mask);
}

__global__ void k_ingest_degree(const uint32_t* __restrict__ off, uint32_t n, uint32_t* __restrict__ deg) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    deg[v] = off[v + 1] - off[v];
}

// Raw random batch, the same draws as the host generator prx_gen_batch:
// deletion i is the first non-self-loop edge among kDelTries uniform draws
// (n, n when all are self-loops: dropped by the tidy); insertion i is a
// uniform pair.
// Edge e of the out-CSR in the compact order (the order of prx_graph_download)
// as (u, v).  With row segments, seg holds each segment's first edge in the
// compact order, then its position in the device array (nseg each).
__device__ __forceinline__ void edge_at(const uint32_t* __restrict__ xoff, const uint32_t* __restrict__ xedg, uint32_t n,
                                        uint32_t shift, uint32_t nseg, const unsigned long long* __restrict__ seg,
                                        uint64_t e, uint32_t& u, uint32_t& v) {
  uint32_t k = 0, r0 = 0, rows = n;
  uint64_t rel = e, at = 0;
  if (nseg > 1) {
    uint32_t lo = 0, hi = nseg - 1;  // last segment whose first edge is <= e
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (seg[mid] <= e) lo = mid;
      else hi = mid - 1;
    }
    k = lo;
    r0 = (uint32_t)((uint64_t)k << shift);
    const uint64_t left = (uint64_t)n - r0, full = 1ull << shift;
    rows = (uint32_t)(left < full ? left : full);
    rel = e - seg[k];
    at = seg[nseg + k];
  }
  const uint32_t* off = xoff + r0 + k;  // the segment's rows + 1 offsets
  uint32_t lo = 0, hi = rows;           // last row whose start is <= rel
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (off[mid] <= rel) lo = mid;
    else hi = mid - 1;
  }
  u = r0 + lo;
  v = xedg[at + rel];
}

__global__ void k_gen_deletions(const uint32_t* __restrict__ xoff, const uint32_t* __restrict__ xedg, uint32_t n,
                                uint64_t m, uint32_t shift, uint32_t nseg, const unsigned long long* __restrict__ seg,
                                uint64_t seed, uint32_t count, uint32_t* __restrict__ du, uint32_t* __restrict__ dv) {
  using namespace prx_hash;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    uint32_t ou = n, ov = n;
    for (uint64_t t = 0; t < kDelTries && m; ++t) {
      const uint64_t e = (rnd(seed, kDelStream, (uint64_t)i * kDelTries + t) >> 11) % m;
      uint32_t u, v;
      edge_at(xoff, xedg, n, shift, nseg, seg, e, u, v);
      if (u == v) continue;
      ou = u;
      ov = v;
      break;
    }
    du[i] = ou;
    dv[i] = ov;
  }
}

__global__ void k_gen_insertions(uint32_t n, uint64_t seed, uint32_t count, uint32_t* __restrict__ iu,
                                 uint32_t* __restrict__ iv) {
  using namespace prx_hash;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const uint64_t h = rnd(seed, kInsStream, i);
    iu[i] = below(h, n);
    iv[i] = below(mix64(h), n);
  }
}

}  // namespace prx

// Device buffers of one tidy call.
struct TidyBufs {
  uint32_t *u = nullptr, *v = nullptr, *flag = nullptr, *pos = nullptr, *hist = nullptr;
  unsigned long long *key = nullptr, *key2 = nullptr;
  void release() { graph_free({u, v, flag, pos, hist, key, key2}); }
};

// Tidy one list (deletions or insertions) of `count` edges already in b.u /
// b.v on the device into host arrays; *kept receives the tidied length.
// Frees every buffer of b.
static int tidy_core(prx_context* c, const GraphDev& g, TidyBufs& b, uint32_t count, bool deletions, uint32_t* ou,
                     uint32_t* ov, uint64_t* kept) {
  cudaStream_t s = c->stream;
  int vbits = 1;
  while (vbits < 32 && (1ull << vbits) < g.n) ++vbits;
  // deletions of a one-segment graph sort by their out-CSR positions (32-bit
  // keys, fewer radix passes); every other list by u * 2^vbits + v
  const int pos_keys = deletions && g.nseg == 1 ? 1 : 0;
  const int key_bits = pos_keys ? 32 : std::min(64, 2 * vbits);
  const uint32_t tiles = (count + kSortTile - 1) / kSortTile;
  auto fail = [&](cudaError_t e) {
    b.release();
    set_error(std::string("prx_graph_tidy_batch: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
  };
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = graph_alloc(&b.flag, 4ull * (count + 1), s);
  if (e == cudaSuccess) e = graph_alloc(&b.pos, 4ull * (count + 1), s);
  if (e == cudaSuccess) e = graph_alloc(&b.hist, 4ull * ((size_t)kRadix * tiles + 1), s);
  if (e == cudaSuccess) e = graph_alloc(&b.key, 8ull * (count + 2), s);   // + 2: radix_sort_u64's slack
  if (e == cudaSuccess) e = graph_alloc(&b.key2, 8ull * (count + 2), s);
  if (e != cudaSuccess) return fail(e);
  const int grid = grid_of(count, c->sms);
  // 1-2. existence and keys, then compaction of the kept keys
  k_tidy_keys<<<grid, 256, 0, s>>>(g.xoff, g.xedg, g.xbase, g.seg_shift, g.n, b.u, b.v, count, deletions ? 1 : 0,
                                   pos_keys, vbits, b.flag, b.key);
  e = cudaMemcpyAsync(b.pos, b.flag, 4ull * count, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.pos + count, 0, 4, s);
  if (e == cudaSuccess) e = exclusive_scan_u32(b.pos, count + 1, s);
  uint32_t m2 = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&m2, b.pos + count, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) k_compact64<<<grid, 256, 0, s>>>(b.key, b.flag, b.pos, count, b.key2);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(e);
  if (m2 == 0) {
    b.release();
    return PRX_OK;
  }
  // 3. radix sort of key2[0 .. m2)
  unsigned long long* src = nullptr;
  e = radix_sort_u64(b.key2, b.key, m2, 0, key_bits, b.hist, c->sms, s, &src);
  if (e != cudaSuccess) return fail(e);
  // 4. unique and decode
  const int g2 = grid_of(m2, c->sms);
  k_first_flags<<<g2, 256, 0, s>>>(src, m2, b.flag);
  e = cudaMemcpyAsync(b.pos, b.flag, 4ull * m2, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.pos + m2, 0, 4, s);
  if (e == cudaSuccess) e = exclusive_scan_u32(b.pos, m2 + 1, s);
  uint32_t m3 = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&m3, b.pos + m2, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    k_decode<<<g2, 256, 0, s>>>(src, b.flag, b.pos, m2, pos_keys, vbits, g.xoff, g.n, g.xedg, b.u, b.v);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && m3) e = cudaMemcpyAsync(ou, b.u, 4ull * m3, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && m3) e = cudaMemcpyAsync(ov, b.v, 4ull * m3, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail(e);
  b.release();
  *kept = m3;
  return PRX_OK;
}

// Tidy one list of `count` edges from host arrays into host arrays.
static int tidy_list(prx_context* c, const GraphDev& g, const uint32_t* hu, const uint32_t* hv, uint64_t count64,
                     bool deletions, uint32_t* ou, uint32_t* ov, uint64_t* kept) {
  *kept = 0;
  if (count64 == 0) return PRX_OK;
  if (count64 > kMaxVertices) FAIL(PRX_ERANGE, "prx_graph_tidy_batch: batch too large");
  const uint32_t count = (uint32_t)count64;
  TidyBufs b;
  cudaError_t e = graph_alloc(&b.u, 4ull * count, c->stream);
  if (e == cudaSuccess) e = graph_alloc(&b.v, 4ull * count, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b.u, hu, 4ull * count, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b.v, hv, 4ull * count, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) {
    b.release();
    set_error(std::string("prx_graph_tidy_batch: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
  }
  return tidy_core(c, g, b, count, deletions, ou, ov, kept);
}

// prx_graph_create_from_edges[_device].  Device memory: the edge arrays (host
// edges only), 3 key buffers of 8 bytes per edge, 2 scan buffers of 4 bytes
// per edge, then the graph.
static int create_from_edges(prx_context* c, uint32_t n, const uint32_t* u, const uint32_t* v, uint64_t count64,
                             int self_loops, bool on_device, prx_graph** out) {
  if (!c || !out) FAIL(PRX_EINVAL, "prx_graph_create_from_edges: NULL context or output");
  *out = nullptr;
  if (count64 && (!u || !v)) FAIL(PRX_EINVAL, "prx_graph_create_from_edges: NULL edge arrays");
  const uint64_t total64 = count64 + (self_loops ? n : 0);
  if (total64 > kMaxVertices)  // 32-bit offsets, and 32-bit grid-stride indices that must not wrap
    FAIL(PRX_ERANGE, "prx_graph_create_from_edges: too many edges (more than 2^32 - 2^24)");
  if (count64 && n == 0) FAIL(PRX_EINVAL, "prx_graph_create_from_edges: edges given with n = 0");
  if (n > kMaxVertices) FAIL(PRX_ERANGE, "prx_graph_create_from_edges: more than 2^32 - 2^24 vertices");
  TRY_CUDA_ST(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const uint32_t count = (uint32_t)count64, total = (uint32_t)total64;
  int vbits = 1;
  while (vbits < 32 && (1ull << vbits) < n) ++vbits;
  prx_graph* gr = new prx_graph();
  gr->ctx = c;
  GraphDev& g = gr->g;
  g.device = c->device;
  g.n = n;
  TidyBufs b;                          // u, v (host edges), flag, pos, hist, key, key2
  unsigned long long* key3 = nullptr;
  uint32_t* bad = nullptr;
  auto release = [&]() {
    b.release();
    b = TidyBufs();
    graph_free({key3, bad});
    key3 = nullptr;
    bad = nullptr;
  };
  auto fail = [&](cudaError_t e) {
    release();
    prx_graph_destroy(gr);
    set_error(std::string("prx_graph_create_from_edges: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
  };
  const size_t cap = total ? total : 1;
  const uint32_t tiles = (total + kSortTile - 1) / kSortTile;
  cudaError_t e = cudaSuccess;
  const uint32_t *du = u, *dv = v;
  if (!on_device && count) {
    if (e == cudaSuccess) e = graph_alloc(&b.u, 4ull * count, s);
    if (e == cudaSuccess) e = graph_alloc(&b.v, 4ull * count, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.u, u, 4ull * count, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.v, v, 4ull * count, cudaMemcpyHostToDevice, s);
    du = b.u;
    dv = b.v;
  }
  if (e == cudaSuccess) e = graph_alloc(&b.flag, 4ull * (cap + 1), s);
  if (e == cudaSuccess) e = graph_alloc(&b.pos, 4ull * (cap + 1), s);
  if (e == cudaSuccess) e = graph_alloc(&b.hist, 4ull * ((size_t)kRadix * tiles + 1), s);
  if (e == cudaSuccess) e = graph_alloc(&b.key, 8ull * (cap + 2), s);    // + 2: radix_sort_u64's slack
  if (e == cudaSuccess) e = graph_alloc(&b.key2, 8ull * (cap + 2), s);
  if (e == cudaSuccess) e = graph_alloc(&key3, 8ull * (cap + 2), s);
  if (e == cudaSuccess) e = graph_alloc(&bad, 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, 4, s);
  if (e != cudaSuccess) return fail(e);
  const int grid = grid_of(cap, c->sms);
  // sorted unique (u, v): the out-CSR
  k_ingest_keys<<<grid, 256, 0, s>>>(du, dv, count, n, self_loops ? 1 : 0, vbits, b.key, bad);
  unsigned long long* sorted = nullptr;
  e = radix_sort_u64(b.key, b.key2, total, 0, 2 * vbits, b.hist, c->sms, s, &sorted);
  if (e != cudaSuccess) return fail(e);
  unsigned long long* uniq = sorted == b.key ? b.key2 : b.key;  // the sort's spare buffer
  k_first_flags<<<grid, 256, 0, s>>>(sorted, total, b.flag);
  e = cudaMemcpyAsync(b.pos, b.flag, 4ull * total, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.pos + total, 0, 4, s);
  if (e == cudaSuccess) e = exclusive_scan_u32(b.pos, total + 1, s);
  uint32_t m = 0, bad_h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&m, b.pos + total, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad_h, bad, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) k_ingest_split<<<grid, 256, 0, s>>>(sorted, b.flag, b.pos, total, vbits, 1, uniq, key3);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(e);
  if (bad_h) {
    release();
    prx_graph_destroy(gr);
    FAIL(PRX_EINVAL, "prx_graph_create_from_edges: vertex id out of range");
  }
  g.m = g.m_cap = m;
  if (e == cudaSuccess) e = graph_alloc(&g.xoff, 4ull * ((size_t)n + 1), s);
  if (e == cudaSuccess) e = graph_alloc(&g.xedg, 4ull * (m ? m : 1), s);
  if (e == cudaSuccess) e = graph_alloc(&g.xtoff, 4ull * ((size_t)n + 1), s);
  if (e == cudaSuccess) e = graph_alloc(&g.xtedg, 4ull * edge_slots(m), s);
  if (e == cudaSuccess) e = graph_alloc(&g.xtdat, 4ull * (n ? n : 1), s);
  if (e != cudaSuccess) return fail(e);
  const int gm = grid_of(m, c->sms), gn = grid_of((uint64_t)n + 1, c->sms);
  k_ingest_offsets<<<gn, 256, 0, s>>>(uniq, m, vbits, n, g.xoff);
  k_ingest_columns<<<gm, 256, 0, s>>>(uniq, m, vbits, g.xedg);
  k_ingest_degree<<<gn, 256, 0, s>>>(g.xoff, n, g.xtdat);
  // the transpose: the swapped keys v * 2^b + u arrive ordered by u, so a
  // stable sort on their high half (v) alone orders them by (v, u); the
  // spare buffer is the old sorted one
  e = radix_sort_u64(key3, sorted, m, vbits, 2 * vbits, b.hist, c->sms, s, &sorted);
  if (e != cudaSuccess) return fail(e);
  k_ingest_offsets<<<gn, 256, 0, s>>>(sorted, m, vbits, n, g.xtoff);
  k_ingest_columns<<<gm, 256, 0, s>>>(sorted, m, vbits, g.xtedg);
  e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  release();
  if (e == cudaSuccess) e = build_classes(g, c->sms, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = tune_apply_cached(g, c->sms, s);
  if (e != cudaSuccess) return fail(e);
  *out = gr;
  return PRX_OK;
}

extern "C" {

int prx_graph_create_from_edges(prx_context* c, uint32_t n, const uint32_t* u, const uint32_t* v, uint64_t count,
                                int self_loops, prx_graph** out) {
  return create_from_edges(c, n, u, v, count, self_loops, false, out);
}

int prx_graph_create_from_edges_device(prx_context* c, uint32_t n, const uint32_t* u, const uint32_t* v,
                                       uint64_t count, int self_loops, prx_graph** out) {
  return create_from_edges(c, n, u, v, count, self_loops, true, out);
}

int prx_graph_tidy_batch(prx_context* c, prx_graph* gr, const uint32_t* du, const uint32_t* dv, uint64_t nd,
                         const uint32_t* iu, const uint32_t* iv, uint64_t ni, uint32_t* out_du, uint32_t* out_dv,
                         uint64_t* out_nd, uint32_t* out_iu, uint32_t* out_iv, uint64_t* out_ni) {
  if (!c || !gr || gr->ctx != c) FAIL(PRX_EINVAL, "prx_graph_tidy_batch: bad context or graph");
  const GraphDev& g = gr->g;
  if (!g.xoff) FAIL(PRX_ESTATE, "prx_graph_tidy_batch: graph has no out-CSR");
  if (!out_nd || !out_ni) FAIL(PRX_EINVAL, "prx_graph_tidy_batch: NULL output length");
  if ((nd && (!du || !dv || !out_du || !out_dv)) || (ni && (!iu || !iv || !out_iu || !out_iv)))
    FAIL(PRX_EINVAL, "prx_graph_tidy_batch: NULL array with a non-zero length");
  for (uint64_t i = 0; i < nd; ++i)
    if (du[i] >= g.n || dv[i] >= g.n) FAIL(PRX_EINVAL, "prx_graph_tidy_batch: deletion vertex id out of range");
  for (uint64_t i = 0; i < ni; ++i)
    if (iu[i] >= g.n || iv[i] >= g.n) FAIL(PRX_EINVAL, "prx_graph_tidy_batch: insertion vertex id out of range");
  TRY_CUDA_ST(cudaSetDevice(c->device));
  int st = tidy_list(c, g, du, dv, nd, true, out_du, out_dv, out_nd);
  if (st) return st;
  return tidy_list(c, g, iu, iv, ni, false, out_iu, out_iv, out_ni);
}

int prx_graph_gen_batch(prx_context* c, prx_graph* gr, uint64_t nd_req, uint64_t ni_req, uint64_t seed,
                        uint32_t* out_du, uint32_t* out_dv, uint64_t* out_nd, uint32_t* out_iu, uint32_t* out_iv,
                        uint64_t* out_ni) {
  if (!c || !gr || gr->ctx != c) FAIL(PRX_EINVAL, "prx_graph_gen_batch: bad context or graph");
  const GraphDev& g = gr->g;
  if (!g.xoff) FAIL(PRX_ESTATE, "prx_graph_gen_batch: graph has no out-CSR");
  if (!out_nd || !out_ni || (nd_req && (!out_du || !out_dv)) || (ni_req && (!out_iu || !out_iv)))
    FAIL(PRX_EINVAL, "prx_graph_gen_batch: NULL output");
  if (g.n == 0) FAIL(PRX_EINVAL, "prx_graph_gen_batch: empty graph");
  if (nd_req > kMaxVertices || ni_req > kMaxVertices) FAIL(PRX_ERANGE, "prx_graph_gen_batch: batch too large");
  TRY_CUDA_ST(cudaSetDevice(c->device));
  *out_nd = *out_ni = 0;
  for (int del = 1; del >= 0; --del) {
    const uint32_t count = (uint32_t)(del ? nd_req : ni_req);
    if (!count) continue;
    TidyBufs b;
    unsigned long long* seg = nullptr;  // row segments: first edges (compact order), then device positions
    cudaError_t e = graph_alloc(&b.u, 4ull * count, c->stream);
    if (e == cudaSuccess) e = graph_alloc(&b.v, 4ull * count, c->stream);
    if (e == cudaSuccess && del && g.nseg > 1) {
      std::vector<unsigned long long> h(2 * (size_t)g.nseg);
      for (uint32_t k = 0; k < g.nseg; ++k) {
        h[k] = g.xseg0[k];
        h[g.nseg + k] = g.xpos[k];
      }
      e = graph_alloc(&seg, 8 * h.size(), c->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(seg, h.data(), 8 * h.size(), cudaMemcpyHostToDevice, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);  // h is about to go
    }
    if (e == cudaSuccess) {
      const int grid = grid_of(count, c->sms);
      if (del)
        k_gen_deletions<<<grid, 256, 0, c->stream>>>(g.xoff, g.xedg, g.n, g.m, g.seg_shift, g.nseg, seg, seed, count,
                                                     b.u, b.v);
      else k_gen_insertions<<<grid, 256, 0, c->stream>>>(g.n, seed, count, b.u, b.v);
      e = cudaGetLastError();
    }
    if (seg) cudaFreeAsync(seg, c->stream);
    if (e != cudaSuccess) {
      b.release();
      set_error(std::string("prx_graph_gen_batch: ") + cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
    }
    const int st = del ? tidy_core(c, g, b, count, true, out_du, out_dv, out_nd)
                       : tidy_core(c, g, b, count, false, out_iu, out_iv, out_ni);
    if (st) return st;
  }
  return PRX_OK;
}

}  // extern "C"
