// prx_batch.cu -- apply a tidied batch update to the device CSRs.
//
// The reference applies a batch on the host, vertex by vertex
// (applyBatchUpdateOmpU, inc/batch.hxx:239-247), and rebuilds the transpose
// from scratch (transposeWithDegreeOmp, inc/transpose.hxx:128-134); both are
// outside its timed region.  Here the update runs on the device:
//   1. check the batch is tidy against the current graph (deletions exist,
//      insertions do not), so the merge below cannot go wrong;
//   2. per-vertex degree deltas and "touched" bitmaps for both CSRs;
//   3. new offsets = exclusive scan of the new degrees (per row segment on
//      graphs with 64-bit offsets, whose segments then move to new bases);
//   4. untouched rows are copied in windows of equal length (coalesced),
//      touched rows are merged by a whole warp each (old row minus
//      deletions, plus insertions, ascending -- the LazyBitset order the
//      reference keeps);
//   5. out-degrees and the in-degree classes are refreshed.
// The in-CSR needs the batch ordered by (v, u); batch_by_target makes that
// order on the device.
#include <algorithm>
#include <vector>
#include "prx_device.cuh"

namespace prx {

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* a, uint32_t len, uint32_t key) {
  uint32_t lo = 0, hi = len;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Does row u (of a CSR with row segments, see GraphDev) hold v?
__device__ __forceinline__ bool row_has(const uint32_t* off, const uint32_t* edg, const unsigned long long* base,
                                        uint32_t shift, uint32_t u, uint32_t v) {
  const uint64_t k = seg_index(u, shift);
  const uint32_t b = off[k], len = off[k + 1] - b;
  const uint32_t* row = seg_edges(edg, base, shift, u) + b;
  const uint32_t i = lower_bound_u32(row, len, v);
  return i < len && row[i] == v;
}

// Flags err if a deletion is missing or an insertion already exists.
__global__ void k_batch_check(const uint32_t* __restrict__ off, const uint32_t* __restrict__ edg,
                              const unsigned long long* __restrict__ base, uint32_t shift,
                              const uint32_t* du, const uint32_t* dv, uint32_t nd,
                              const uint32_t* iu, const uint32_t* iv, uint32_t ni, uint32_t* err) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd + ni; i += gridDim.x * blockDim.x) {
    const bool del = i < nd;
    const uint32_t u = del ? du[i] : iu[i - nd], v = del ? dv[i] : iv[i - nd];
    if (row_has(off, edg, base, shift, u, v) != del) atomicOr(err, del ? 1u : 2u);
  }
}

// Per-vertex degree deltas and touched bits of both CSRs; with row segments
// (segd not null) also each segment's edge-count delta, out-CSR segments
// (by u) first, then in-CSR segments (by v).
__global__ void k_batch_deltas(const uint32_t* du, const uint32_t* dv, uint32_t nd,
                               const uint32_t* iu, const uint32_t* iv, uint32_t ni,
                               int32_t* dout, int32_t* din, uint32_t* tout, uint32_t* tin,
                               uint32_t shift, uint32_t nseg, long long* segd) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd + ni; i += gridDim.x * blockDim.x) {
    const bool del = i < nd;
    const uint32_t u = del ? du[i] : iu[i - nd], v = del ? dv[i] : iv[i - nd];
    atomicAdd(dout + u, del ? -1 : 1);
    atomicAdd(din + v, del ? -1 : 1);
    atomicOr(tout + (u >> 5), 1u << (u & 31));
    atomicOr(tin + (v >> 5), 1u << (v & 31));
    if (segd) {  // two's complement sums in unsigned words
      const unsigned long long one = del ? ~0ull : 1ull;
      atomicAdd(reinterpret_cast<unsigned long long*>(segd) + ((uint64_t)u >> shift), one);
      atomicAdd(reinterpret_cast<unsigned long long*>(segd) + nseg + ((uint64_t)v >> shift), one);
    }
  }
}

// New degrees laid out like the offsets (row v at seg_index(v), a 0 closing
// each row segment), so one exclusive scan per segment gives its offsets.
__global__ void k_new_degree(const uint32_t* __restrict__ off, const int32_t* __restrict__ delta, uint32_t n,
                             uint32_t shift, uint64_t entries, uint32_t* __restrict__ deg) {
  const uint64_t per = (shift >= 32 ? (uint64_t)n : (1ull << shift)) + 1;  // entries of a full segment
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < entries;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = i / per, j = i - k * per;
    const uint64_t v = (shift >= 32 ? 0 : (k << shift)) + j;
    const bool row = j + 1 < per && v < n;
    deg[i] = row ? (uint32_t)((int64_t)(off[i + 1] - off[i]) + delta[v]) : 0u;
  }
}

// Rows keyed by `key` (u for the out-CSR, v for the in-CSR); deletions and
// insertions sorted by (key, val).
//
// Untouched rows keep their ids, and a run of untouched rows between two
// touched ones is one contiguous block in the old edge array and in the new
// one, shifted by a constant: k_copy_runs copies the runs as shifted blocks,
// warps taking windows of kWindow old positions (equal work whatever the row
// lengths), each finding the run under its window's start with a 32-way
// search over the touched-row list.
//
// A touched row is merged by ranks, each id on its own: a kept old id w goes
// to (its index) - (deleted ids below w) + (inserted ids below w); an
// inserted id x goes to (its index among the row's insertions) + (old ids
// below x) - (deleted ids below x).  The batch is tidy (deletions are old
// ids, insertions are not), so these are the positions of the sorted merge;
// every lane finds its own with binary searches, a warp takes a row, and hub
// rows with 100k ids are cut into pieces for all warps.
// One touched row's merge, element by element: old id j of the row and
// inserted id k land at independent positions, so a row can be split among
// any number of warps.
struct RowMerge {
  const uint32_t* old;   // the row's old ids
  const uint32_t* del;   // its deletions, ascending (a subset of old)
  const uint32_t* ins;   // its insertions, ascending (none in old)
  uint32_t len, nd, ni;
  uint32_t* out;         // the row's new ids
  __device__ __forceinline__ void old_id(uint32_t j) const {
    const uint32_t w = old[j];
    const uint32_t p = lower_bound_u32(del, nd, w);  // deleted ids below w: all of them precede w
    if (p < nd && del[p] == w) return;
    out[j - p + lower_bound_u32(ins, ni, w)] = w;
  }
  __device__ __forceinline__ void ins_id(uint32_t k) const {
    const uint32_t x = ins[k];
    out[k + lower_bound_u32(old, len, x) - lower_bound_u32(del, nd, x)] = x;
  }
};

__device__ __forceinline__ RowMerge row_merge(const uint32_t* oedg, uint32_t* nedg, uint32_t os, uint32_t len,
                                              uint32_t ns, const uint32_t* dv, uint32_t d0, uint32_t d1,
                                              const uint32_t* iv, uint32_t i0, uint32_t i1) {
  return RowMerge{oedg + os, dv + d0, iv + i0, len, d1 - d0, i1 - i0, nedg + ns};
}

// Per row, the range of its entries in a batch list sorted by row
// (begin / end zeroed beforehand; rows without entries keep [0, 0)).
__global__ void k_batch_ranges(const uint32_t* __restrict__ key, uint32_t count, uint32_t* __restrict__ begin,
                               uint32_t* __restrict__ end) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const uint32_t k = key[i];
    if (i == 0 || key[i - 1] != k) begin[k] = i;
    if (i + 1 == count || key[i + 1] != k) end[k] = i + 1;
  }
}

constexpr uint32_t kWindow = 16384;

// Touched rows as an ascending list: per bitmap word its popcount (a 0 after
// the last word, for the scan), then the ids at the scanned positions.
__global__ void k_word_pop(const uint32_t* __restrict__ t, uint32_t words, uint32_t* __restrict__ cnt) {
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w <= words; w += gridDim.x * blockDim.x)
    cnt[w] = w < words ? (uint32_t)__popc(t[w]) : 0u;
}
__global__ void k_touched_list(const uint32_t* __restrict__ t, uint32_t words, const uint32_t* __restrict__ pos,
                               uint32_t* __restrict__ list) {
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += gridDim.x * blockDim.x) {
    uint32_t i = pos[w];
    for (uint32_t b = t[w]; b; b &= b - 1) list[i++] = (w << 5) | (uint32_t)(__ffs(b) - 1);
  }
}

// One CSR (or one row segment of it): rows [0, rows) with old offsets ooff
// (rows + 1 entries, relative to oedg) and new offsets noff (relative to
// nedg); trow[0 .. T): its touched rows, ascending, as rbase + row.  Run j
// (j <= T) is the untouched rows between touched rows j-1 and j.
struct Runs {
  const uint32_t* ooff;
  const uint32_t* noff;
  const uint32_t* trow;
  uint32_t T, rows, rbase;
  const uint32_t* Tp;  // not null: T is read here on the device (the multi-batch solve)
  __device__ __forceinline__ void load_T() {
    if (Tp) T = *Tp;
  }
  __device__ __forceinline__ uint32_t first(uint32_t j) const { return j ? trow[j - 1] - rbase + 1 : 0u; }
  __device__ __forceinline__ uint32_t end(uint32_t j) const { return j < T ? trow[j] - rbase : rows; }
};

__global__ void __launch_bounds__(kThreads) k_copy_runs(Runs r, const uint32_t* __restrict__ oedg,
                                                        uint32_t* __restrict__ nedg) {
  r.load_T();
  const uint32_t lane = lane_id();
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  // old positions [start, end): a CSR's offsets start at 0, a layout chunk's where its region starts
  const uint32_t start = r.ooff[0], end = r.ooff[r.rows];
  const uint32_t windows = (uint32_t)(((uint64_t)(end - start) + kWindow - 1) / kWindow);
  for (uint32_t wi = warp; wi < windows; wi += nwarps) {
    const uint32_t p0 = start + wi * kWindow, p1 = (uint32_t)min((uint64_t)end, (uint64_t)p0 + kWindow);
    // the last run starting at or before p0 (run 0 starts at `start`)
    uint32_t lo = 0, hi = r.T + 1;
    while (hi - lo > 1) {
      const uint32_t step = (hi - lo + 31) / 32, j = lo + lane * step;
      const bool ok = j < hi && r.ooff[r.first(j)] <= p0;
      const unsigned bal = __ballot_sync(0xffffffffu, ok);
      lo += (31u - __clz(bal)) * step;
      hi = min(hi, lo + step);
    }
    for (uint32_t j = lo; j <= r.T; ++j) {
      const uint32_t a = r.first(j), s0 = r.ooff[a];
      if (s0 >= p1) break;
      const uint32_t lo_p = max(p0, s0), hi_p = min(p1, r.ooff[r.end(j)]);
      const uint32_t shift = r.noff[a] - s0;  // new position - old position (mod 2^32)
      for (uint32_t base = lo_p; base < hi_p; base += 256) {  // 8 ids per lane in flight
        uint32_t val[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const uint32_t pq = base + 32u * q + lane;
          val[q] = pq < hi_p ? oedg[pq] : 0u;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const uint32_t pq = base + 32u * q + lane;
          if (pq < hi_p) nedg[pq + shift] = val[q];
        }
      }
    }
  }
}

// The touched rows, one warp each; rows of more than kBigRow ids (old and
// inserted) are listed for k_merge_big instead: entry i of big[] holds the
// row's place in the touched list and the number of 1024-id pieces of the
// rows listed before it, both from one 64-bit atomic (pieces in the high
// word, rows in the low one), so the pieces are numbered in list order.
constexpr uint32_t kBigRow = 4096;
constexpr uint32_t kPiece = 1024;

__device__ __forceinline__ RowMerge touched_merge(const Runs& r, uint32_t i, const uint32_t* oedg, uint32_t* nedg,
                                                  const uint32_t* dv, const uint32_t* dbeg, const uint32_t* dend,
                                                  const uint32_t* iv, const uint32_t* ibeg, const uint32_t* iend) {
  const uint32_t row = r.trow[i] - r.rbase;
  const uint32_t s = r.ooff[row], e = r.ooff[row + 1];
  return row_merge(oedg, nedg, s, e - s, r.noff[row], dv, dbeg[row], dend[row], iv, ibeg[row], iend[row]);
}

__device__ __forceinline__ uint32_t merge_pieces(const RowMerge& m) {
  return (m.len + kPiece - 1) / kPiece + (m.ni + kPiece - 1) / kPiece;
}

__global__ void __launch_bounds__(kThreads) k_merge_touched(Runs r, const uint32_t* __restrict__ oedg,
                                                            uint32_t* __restrict__ nedg, const uint32_t* dv,
                                                            const uint32_t* __restrict__ dbeg,
                                                            const uint32_t* __restrict__ dend, const uint32_t* iv,
                                                            const uint32_t* __restrict__ ibeg,
                                                            const uint32_t* __restrict__ iend, uint32_t* big,
                                                            unsigned long long* nbig) {
  r.load_T();
  const uint32_t lane = lane_id();
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = warp; i < r.T; i += nwarps) {
    const RowMerge m = touched_merge(r, i, oedg, nedg, dv, dbeg, dend, iv, ibeg, iend);
    if (m.len + m.ni > kBigRow) {
      if (lane == 0) {
        const unsigned long long old = atomicAdd(nbig, ((unsigned long long)merge_pieces(m) << 32) | 1ull);
        const uint32_t slot = (uint32_t)old;
        big[2 * slot] = i;
        big[2 * slot + 1] = (uint32_t)(old >> 32);
      }
      continue;
    }
    for (uint32_t j = lane; j < m.len; j += 32) m.old_id(j);
    for (uint32_t k = lane; k < m.ni; k += 32) m.ins_id(k);
  }
}

// The pieces of the long touched rows, one warp each: warp p finds its row as
// the last listed one whose first piece is at or before p.
__global__ void __launch_bounds__(kThreads) k_merge_big(Runs r, const uint32_t* __restrict__ oedg,
                                                        uint32_t* __restrict__ nedg, const uint32_t* dv,
                                                        const uint32_t* __restrict__ dbeg,
                                                        const uint32_t* __restrict__ dend, const uint32_t* iv,
                                                        const uint32_t* __restrict__ ibeg,
                                                        const uint32_t* __restrict__ iend,
                                                        const uint32_t* __restrict__ big,
                                                        const unsigned long long* __restrict__ nbig) {
  const uint32_t lane = lane_id();
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const unsigned long long tally = *nbig;
  const uint32_t rows = (uint32_t)tally, pieces = (uint32_t)(tally >> 32);
  for (uint32_t p = warp; p < pieces; p += nwarps) {
    uint32_t lo = 0, hi = rows;  // big[2*lo+1] <= p < big[2*hi+1]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (big[2 * mid + 1] <= p) lo = mid; else hi = mid;
    }
    const RowMerge m = touched_merge(r, big[2 * lo], oedg, nedg, dv, dbeg, dend, iv, ibeg, iend);
    const uint32_t c = p - big[2 * lo + 1], po = (m.len + kPiece - 1) / kPiece;
    if (c < po) {
      for (uint32_t j = c * kPiece + lane; j < min(m.len, (c + 1) * kPiece); j += 32) m.old_id(j);
    } else {
      const uint32_t c2 = c - po;
      for (uint32_t k = c2 * kPiece + lane; k < min(m.ni, (c2 + 1) * kPiece); k += 32) m.ins_id(k);
    }
  }
}

// ---- LOW layouts carried to the new version ---------------------------------
// A cached layout (see ChunkLayout) of the old version becomes the new
// version's without a rebuild: rows the batch did not touch keep their chunk
// counts and segments (copied as shifted runs by k_copy_runs), touched rows
// are counted and scattered again from the new in-CSR (a row that crossed
// the LOW bound gains or loses its segments), with the same hot numbering.

// New chunk counts (K x (n + 1), a 0 closing each chunk row): untouched rows
// from the old offsets, touched rows from their new in-edges if still LOW.
__global__ void k_layout_counts(const uint32_t* __restrict__ lay_off, const uint32_t* __restrict__ xtoff,
                                const uint32_t* __restrict__ xtedg, const uint32_t* __restrict__ touched,
                                uint32_t n, uint32_t width, int K, uint32_t* __restrict__ cnt) {
  const size_t row = (size_t)n + 1;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x) {
    if (v == n) {
      for (int k = 0; k < K; ++k) cnt[k * row + n] = 0;
      continue;
    }
    if (!((touched[v >> 5] >> (v & 31u)) & 1u)) {
      for (int k = 0; k < K; ++k) cnt[k * row + v] = lay_off[k * row + v + 1] - lay_off[k * row + v];
      continue;
    }
    uint32_t j = xtoff[v];
    const uint32_t e = xtoff[v + 1];
    const bool low = e - j <= kLowMax;
    for (int k = 0; k < K; ++k) {
      const uint64_t hi = (uint64_t)(k + 1) * width;
      const uint32_t b = j;
      while (low && j < e && xtedg[j] < hi) ++j;
      cnt[k * row + v] = j - b;
    }
  }
}

// The touched rows' segments, a thread per row (at most kLowMax ids).
__global__ void k_layout_touched(const uint32_t* __restrict__ xtoff, const uint32_t* __restrict__ xtedg,
                                 const uint32_t* __restrict__ trow, uint32_t T, const uint32_t* Tp, uint32_t n,
                                 uint32_t width, int K, const uint32_t* __restrict__ off,
                                 uint32_t* __restrict__ edg, const uint32_t* __restrict__ hot_idx,
                                 uint32_t hot_words) {
  const size_t row = (size_t)n + 1;
  if (Tp) T = *Tp;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < T; i += gridDim.x * blockDim.x) {
    const uint32_t v = trow[i];
    uint32_t j = xtoff[v];
    const uint32_t e = xtoff[v + 1];
    if (e - j > kLowMax) continue;
    for (int k = 0; k < K; ++k) {
      const uint64_t hi = (uint64_t)(k + 1) * width;
      uint32_t pos = off[k * row + v];
      while (j < e && xtedg[j] < hi) edg[pos++] = layout_id(hot_idx, hot_words, xtedg[j++]);
    }
  }
}

cudaError_t carry_layout(const ChunkLayout& l, const uint32_t* xtoff, const uint32_t* xtedg, uint32_t n,
                         const uint32_t* touched, const uint32_t* trow, uint32_t T, const uint32_t* Tp,
                         const uint32_t* hot_idx, uint32_t* new_off, uint32_t* new_edg, uint32_t* scan_ws, int sms,
                         cudaStream_t s) {
  const size_t row = (size_t)n + 1, len = (size_t)l.K * row;
  const int grid = sms * 8;
  k_layout_counts<<<grid, kThreads, 0, s>>>(l.off, xtoff, xtedg, touched, n, l.width, l.K, new_off);
  cudaError_t e = exclusive_scan_u32_ws(new_off, (uint32_t)len, scan_ws, s);
  if (e != cudaSuccess) return e;
  for (int k = 0; k < l.K; ++k) {
    const Runs r{l.off + k * row, new_off + k * row, trow, T, n, 0, Tp};
    k_copy_runs<<<grid, kThreads, 0, s>>>(r, l.edg, new_edg);
  }
  if (T || Tp)
    k_layout_touched<<<grid, kThreads, 0, s>>>(xtoff, xtedg, trow, T, Tp, n, l.width, l.K, new_off, new_edg,
                                               l.hot ? hot_idx : nullptr, (n + 31) / 32);
  return cudaGetLastError();
}

// Per row segment k, the slice [lo, hi) of the touched list holding its rows.
__global__ void k_list_slices(const uint32_t* __restrict__ list, uint32_t T, uint32_t n, uint32_t shift,
                              uint32_t nseg, uint32_t* __restrict__ bounds) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= nseg; k += gridDim.x * blockDim.x) {
    const uint64_t v = k == nseg ? (uint64_t)n : (uint64_t)k << shift;
    uint32_t lo = 0, hi = T;  // first entry >= v
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (list[mid] < v) lo = mid + 1; else hi = mid;
    }
    bounds[k] = lo;
  }
}

__global__ void k_out_degree(const uint32_t* __restrict__ off, uint32_t shift, uint32_t n, uint32_t* __restrict__ deg) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    deg[v] = row_len(off, shift, v);
}

__global__ void k_target_keys(const uint32_t* __restrict__ u, const uint32_t* __restrict__ v, uint32_t count,
                              unsigned long long* __restrict__ key) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    key[i] = ((unsigned long long)v[i] << 32) | u[i];
}

__global__ void k_target_split(const unsigned long long* __restrict__ key, uint32_t count, uint32_t* __restrict__ tk,
                               uint32_t* __restrict__ tv) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    tk[i] = (uint32_t)(key[i] >> 32);
    tv[i] = (uint32_t)key[i];
  }
}

cudaError_t batch_by_target(const uint32_t* u, const uint32_t* v, uint32_t count, uint32_t n, uint32_t* tk,
                            uint32_t* tv, int sms, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  int vbits = 1;
  while (vbits < 32 && (1ull << vbits) < n) ++vbits;
  unsigned long long *key = nullptr, *tmp = nullptr, *sorted = nullptr;
  uint32_t* hist = nullptr;
  cudaError_t e = graph_alloc(&key, 8ull * (count + 2), s);
  if (e == cudaSuccess) e = graph_alloc(&tmp, 8ull * (count + 2), s);
  if (e == cudaSuccess) e = graph_alloc(&hist, 4 * radix_hist_words(count), s);
  const int grid = sms * 4;
  if (e == cudaSuccess) k_target_keys<<<grid, kThreads, 0, s>>>(u, v, count, key);
  // the lists are sorted by (u, v): a stable sort on v alone orders them by (v, u)
  if (e == cudaSuccess) e = radix_sort_u64(key, tmp, count, 32, 32 + vbits, hist, sms, s, &sorted);
  if (e == cudaSuccess) k_target_split<<<grid, kThreads, 0, s>>>(sorted, count, tk, tv);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaFreeAsync(key, s);
  cudaFreeAsync(tmp, s);
  cudaFreeAsync(hist, s);
  return e;
}

#define PRX_CU(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { err = e_; goto done; } } while (0)

// Segment layout of one CSR after a batch: first edge of every row segment in
// the compact order (seg0) and in the device array (pos, rounded up to 16
// bytes), and the edge slots to allocate.  cnt: the segments' edge counts.
static uint64_t layout_segments(const std::vector<uint64_t>& cnt, std::vector<uint64_t>& seg0,
                                std::vector<uint64_t>& pos) {
  const size_t k = cnt.size();
  seg0.assign(k, 0);
  pos.assign(k, 0);
  uint64_t compact = 0, slots = 0;
  for (size_t i = 0; i < k; ++i) {
    seg0[i] = compact;
    pos[i] = (slots + 3) & ~3ull;
    compact += cnt[i];
    slots = pos[i] + cnt[i];
  }
  return ((slots + 3) & ~3ull) + 4;
}

// b: device array [du | dv | iu | iv | tdk | tdv | tik | tiv] where the t*
// arrays are the batch sorted by (v, u).  Returns cudaErrorInvalidValue if the
// batch is not tidy for the current graph, cudaErrorInvalidConfiguration if a
// row segment would reach 2^32 edges (nothing is modified in either case).
cudaError_t apply_batch_device(GraphDev& g, const uint32_t* b, uint64_t nd64, uint64_t ni64,
                               int sms, cudaStream_t s) {
  cudaError_t err = cudaSuccess;
  const uint32_t n = g.n, nd = (uint32_t)nd64, ni = (uint32_t)ni64;
  const uint32_t *du = b, *dv = b + nd, *iu = b + 2 * (size_t)nd, *iv = iu + ni;
  const uint32_t *tdk = iv + ni, *tdv = tdk + nd, *tik = tdv + nd, *tiv = tik + ni;
  const uint64_t m2 = g.m - nd + ni;
  const uint32_t words = (n + 31) / 32;
  const uint32_t S = g.seg_shift, nseg = g.nseg;
  const bool segmented = nseg > 1;
  const uint64_t entries = (uint64_t)n + nseg;
  const int grid = sms * 8;
  uint32_t *scratch = nullptr, *noff = nullptr, *ntoff = nullptr, *nedg = nullptr, *ntedg = nullptr, *ndat = nullptr;
  uint32_t *ranges = nullptr, *lists = nullptr;
  const uint32_t* in_list = nullptr;  // the in-CSR's touched rows (plain graphs)
  uint32_t in_T = 0;
  struct NewLayout {
    ChunkLayout* l;
    uint32_t *off, *edg;
  };
  std::vector<NewLayout> layouts_new;
  unsigned long long *nbase = nullptr, *ntbase = nullptr;
  long long* segd = nullptr;
  int32_t *dout, *din;
  uint32_t *tout, *tin, *flag;
  uint32_t hflag = 0;
  // new segment layouts (one segment: the plain CSR)
  std::vector<uint64_t> seg0[2], pos[2];
  uint64_t slots[2] = {m2 ? m2 : 1, edge_slots(m2)};
  // scratch: deltas (2n) + touched (2 words) + flag
  PRX_CU(graph_alloc(&scratch, sizeof(uint32_t) * (2 * (size_t)n + 2 * (size_t)words + 1), s));
  dout = (int32_t*)scratch; din = dout + n;
  tout = (uint32_t*)(din + n); tin = tout + words; flag = tin + words;
  PRX_CU(cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * (2 * (size_t)n + 2 * (size_t)words + 1), s));
  if (segmented) {
    PRX_CU(graph_alloc(&segd, sizeof(long long) * 2 * (size_t)nseg, s));
    PRX_CU(cudaMemsetAsync(segd, 0, sizeof(long long) * 2 * (size_t)nseg, s));
  }
  if (nd + ni) {
    k_batch_check<<<grid, kThreads, 0, s>>>(g.xoff, g.xedg, g.xbase, S, du, dv, nd, iu, iv, ni, flag);
    PRX_CU(cudaMemcpyAsync(&hflag, flag, 4, cudaMemcpyDeviceToHost, s));
    PRX_CU(cudaStreamSynchronize(s));
    if (hflag) { err = cudaErrorInvalidValue; goto done; }
    k_batch_deltas<<<grid, kThreads, 0, s>>>(du, dv, nd, iu, iv, ni, dout, din, tout, tin, S, nseg, segd);
  }
  if (segmented) {  // each segment's new edge count must stay below 2^32
    std::vector<long long> hd(2 * (size_t)nseg);
    PRX_CU(cudaMemcpyAsync(hd.data(), segd, sizeof(long long) * 2 * (size_t)nseg, cudaMemcpyDeviceToHost, s));
    PRX_CU(cudaStreamSynchronize(s));
    for (int csr = 0; csr < 2; ++csr) {
      const std::vector<uint64_t>& old0 = csr ? g.xtseg0 : g.xseg0;
      std::vector<uint64_t> cnt(nseg);
      for (uint32_t k = 0; k < nseg; ++k) {
        const uint64_t oc = (k + 1 < nseg ? old0[k + 1] : g.m) - old0[k];
        const long long c2 = (long long)oc + hd[(size_t)csr * nseg + k];
        if (c2 < 0 || (uint64_t)c2 >= 0xfffffff8ull) { err = cudaErrorInvalidConfiguration; goto done; }
        cnt[k] = (uint64_t)c2;
      }
      slots[csr] = layout_segments(cnt, seg0[csr], pos[csr]);
    }
    PRX_CU(graph_alloc(&nbase, 8 * (size_t)nseg, s));
    PRX_CU(graph_alloc(&ntbase, 8 * (size_t)nseg, s));
    PRX_CU(cudaMemcpyAsync(nbase, pos[0].data(), 8 * (size_t)nseg, cudaMemcpyHostToDevice, s));
    PRX_CU(cudaMemcpyAsync(ntbase, pos[1].data(), 8 * (size_t)nseg, cudaMemcpyHostToDevice, s));
  }
  PRX_CU(graph_alloc(&noff, sizeof(uint32_t) * entries, s));
  PRX_CU(graph_alloc(&ntoff, sizeof(uint32_t) * entries, s));
  PRX_CU(graph_alloc(&nedg, sizeof(uint32_t) * slots[0], s));
  PRX_CU(graph_alloc(&ntedg, sizeof(uint32_t) * slots[1], s));
  PRX_CU(graph_alloc(&ndat, sizeof(uint32_t) * (n ? n : 1), s));
  k_new_degree<<<grid, kThreads, 0, s>>>(g.xoff, dout, n, S, entries, noff);
  k_new_degree<<<grid, kThreads, 0, s>>>(g.xtoff, din, n, S, entries, ntoff);
  for (uint32_t k = 0; k < nseg; ++k) {  // offsets of each segment, relative to its first edge
    const uint64_t v0 = segmented ? (uint64_t)k << S : 0;
    const uint64_t v1 = segmented ? std::min<uint64_t>(n, v0 + (1ull << S)) : n;
    PRX_CU(exclusive_scan_u32(noff + v0 + k, v1 - v0 + 1, s));
    PRX_CU(exclusive_scan_u32(ntoff + v0 + k, v1 - v0 + 1, s));
  }
  // each CSR: its touched rows as a list, the per-row ranges of its deletions
  // and insertions, then the copy of the untouched runs and the merge of the
  // touched rows, segment by segment
  PRX_CU(graph_alloc(&ranges, sizeof(uint32_t) * 4 * (size_t)(n ? n : 1), s));
  PRX_CU(graph_alloc(&lists, sizeof(uint32_t) * ((size_t)words + 2 + 3 * ((size_t)nd + ni) + (size_t)nseg + 4), s));
  {
    uint32_t *dbeg = ranges, *dend = dbeg + n, *ibeg = dend + n, *iend = ibeg + n;
    uint32_t *cnt = lists, *trow = cnt + words + 2, *big = trow + nd + ni, *bounds = big + 2 * ((size_t)nd + ni);
    // 8-byte aligned: the list starts at a graph allocation, and 2 + words + 3(nd + ni) + nseg + 1 is rounded up
    unsigned long long* nbig =
        reinterpret_cast<unsigned long long*>(lists + ((words + 2 + 3 * ((size_t)nd + ni) + nseg + 1 + 1) & ~(size_t)1));
    const uint32_t* keys[2][2] = {{du, iu}, {tdk, tik}};
    const uint32_t* vals[2][2] = {{dv, iv}, {tdv, tiv}};
    const uint32_t* ooff[2] = {g.xoff, g.xtoff};
    const uint32_t* oedg[2] = {g.xedg, g.xtedg};
    const uint32_t* nof[2] = {noff, ntoff};
    uint32_t* ned[2] = {nedg, ntedg};
    const uint32_t* tch[2] = {tout, tin};
    const std::vector<uint64_t>* opos[2] = {&g.xpos, &g.xtpos};
    std::vector<uint32_t> hb(nseg + 1);
    for (int csr = 0; csr < 2; ++csr) {
      uint32_t T = 0;
      if (csr == 1) in_list = trow;
      k_word_pop<<<grid, kThreads, 0, s>>>(tch[csr], words, cnt);
      PRX_CU(exclusive_scan_u32(cnt, words + 1, s));
      PRX_CU(cudaMemcpyAsync(&T, cnt + words, 4, cudaMemcpyDeviceToHost, s));
      k_touched_list<<<grid, kThreads, 0, s>>>(tch[csr], words, cnt, trow);
      PRX_CU(cudaStreamSynchronize(s));  // T
      if (csr == 1) in_T = T;
      k_list_slices<<<(nseg + 256) / 256, 256, 0, s>>>(trow, T, n, S, nseg, bounds);
      PRX_CU(cudaMemcpyAsync(hb.data(), bounds, 4 * ((size_t)nseg + 1), cudaMemcpyDeviceToHost, s));
      PRX_CU(cudaMemsetAsync(ranges, 0, sizeof(uint32_t) * 4 * (size_t)n, s));
      if (nd) k_batch_ranges<<<grid, kThreads, 0, s>>>(keys[csr][0], nd, dbeg, dend);
      if (ni) k_batch_ranges<<<grid, kThreads, 0, s>>>(keys[csr][1], ni, ibeg, iend);
      PRX_CU(cudaStreamSynchronize(s));
      for (uint32_t k = 0; k < nseg; ++k) {
        const uint32_t v0 = segmented ? (uint32_t)((uint64_t)k << S) : 0;
        const uint32_t v1 = segmented ? (uint32_t)std::min<uint64_t>(n, (uint64_t)v0 + (1ull << S)) : n;
        const uint64_t op = segmented ? (*opos[csr])[k] : 0, np = segmented ? pos[csr][k] : 0;
        const Runs r{ooff[csr] + v0 + k, nof[csr] + v0 + k, trow + hb[k], hb[k + 1] - hb[k], v1 - v0, v0, nullptr};
        k_copy_runs<<<grid, kThreads, 0, s>>>(r, oedg[csr] + op, ned[csr] + np);
        if (r.T) {
          PRX_CU(cudaMemsetAsync(nbig, 0, 8, s));
          k_merge_touched<<<grid, kThreads, 0, s>>>(r, oedg[csr] + op, ned[csr] + np, vals[csr][0], dbeg + v0,
                                                    dend + v0, vals[csr][1], ibeg + v0, iend + v0, big, nbig);
          k_merge_big<<<grid, kThreads, 0, s>>>(r, oedg[csr] + op, ned[csr] + np, vals[csr][0], dbeg + v0, dend + v0,
                                                vals[csr][1], ibeg + v0, iend + v0, big, nbig);
        }
      }
    }
  }
  k_out_degree<<<grid, kThreads, 0, s>>>(noff, S, n, ndat);
  // the cached LOW layouts follow the new version (plain graphs; the hot
  // numbering is kept with them)
  if (!segmented) {
    const uint64_t low_edges = g.cls_edges[LOW];
    for (auto& l : g.lay) {
      if (!l.width || !l.off || !l.seg_off.empty()) continue;
      const size_t len = (size_t)l.K * ((size_t)n + 1);
      uint32_t *lo = nullptr, *le = nullptr, *ws = nullptr;
      cudaError_t el = graph_alloc(&lo, sizeof(uint32_t) * len, s);
      if (el == cudaSuccess) el = graph_alloc(&le, sizeof(uint32_t) * edge_slots(low_edges + ni), s);
      if (el == cudaSuccess) el = graph_alloc(&ws, sizeof(uint32_t) * scan_ws_words((uint32_t)len), s);
      if (el == cudaSuccess)
        el = carry_layout(l, ntoff, ntedg, n, tin, in_list, in_T, nullptr, g.hot_idx, lo, le, ws, sms, s);
      if (ws) cudaFreeAsync(ws, s);
      if (el != cudaSuccess) {
        graph_free({lo, le});
        err = el;
        goto done;
      }
      layouts_new.push_back({&l, lo, le});
    }
  }
  PRX_CU(cudaGetLastError());
  PRX_CU(cudaStreamSynchronize(s));
  for (auto& x : layouts_new) {
    graph_free({x.l->off, x.l->edg});
    x.l->off = x.off;
    x.l->edg = x.edg;
  }
  layouts_new.clear();
  graph_free({g.xoff, g.xedg, g.xtoff, g.xtedg, g.xtdat, g.xbase, g.xtbase});
  g.xoff = noff; g.xedg = nedg; g.xtoff = ntoff; g.xtedg = ntedg; g.xtdat = ndat;
  g.xbase = nbase; g.xtbase = ntbase;
  noff = nedg = ntoff = ntedg = ndat = nullptr;
  nbase = ntbase = nullptr;
  if (segmented) {
    g.xseg0 = seg0[0]; g.xpos = pos[0];
    g.xtseg0 = seg0[1]; g.xtpos = pos[1];
  }
  g.m = m2;
  g.m_cap = m2;
  PRX_CU(build_classes(g, sms, s, !segmented));
done:
  for (auto& x : layouts_new) graph_free({x.off, x.edg});
  if (scratch) cudaFreeAsync(scratch, s);
  if (ranges) cudaFreeAsync(ranges, s);
  if (lists) cudaFreeAsync(lists, s);
  if (segd) cudaFreeAsync(segd, s);
  graph_free({noff, ntoff, nedg, ntedg, ndat});
  graph_free({nbase, ntbase});
  return err;
}

// ---- the same apply without host synchronisation or allocation -------------
// (captured into the multi-batch solve's CUDA graph; plain CSRs only)

size_t ApplyWs::words(uint32_t n, uint32_t bmax) {
  const size_t w = ((size_t)n + 31) / 32;
  return 2 * (size_t)n + 2 * w + 4 * (size_t)n + (w + 2) + 3 * (size_t)bmax + 4 + scan_ws_words(n + 1) +
         scan_ws_words((uint32_t)w + 1) + 2;
}

ApplyWs::ApplyWs(uint32_t* base, uint32_t n, uint32_t bmax) {
  const size_t w = ((size_t)n + 31) / 32;
  uint32_t* p = base;
  delta = reinterpret_cast<int32_t*>(p); p += 2 * (size_t)n;
  touched = p; p += 2 * w;
  ranges = p; p += 4 * (size_t)n;
  cnt = p; p += w + 2;
  trow = p; p += bmax;
  big = p; p += 2 * (size_t)bmax;
  if ((p - base) & 1) ++p;  // 8-byte aligned (base is a graph allocation)
  nbig = reinterpret_cast<unsigned long long*>(p); p += 4;
  scan_off = p; p += scan_ws_words(n + 1);
  scan_cnt = p;
}

cudaError_t apply_batch_graph(const CsrSet& src, const CsrSet& dst, uint32_t n, const uint32_t* b, uint32_t nd,
                              uint32_t ni, const ApplyWs& w, int sms, cudaStream_t s) {
  const uint32_t *du = b, *dv = b + nd, *iu = b + 2 * (size_t)nd, *iv = iu + ni;
  const uint32_t *tdk = iv + ni, *tdv = tdk + nd, *tik = tdv + nd, *tiv = tik + ni;
  const uint32_t words = (n + 31) / 32;
  const int grid = sms * 8;
  int32_t *dout = w.delta, *din = w.delta + n;
  uint32_t *tout = w.touched, *tin = w.touched + words;
  cudaError_t e = cudaMemsetAsync(w.delta, 0, sizeof(uint32_t) * (2 * (size_t)n + 2 * (size_t)words), s);
  if (e != cudaSuccess) return e;
  if (nd + ni) k_batch_deltas<<<grid, kThreads, 0, s>>>(du, dv, nd, iu, iv, ni, dout, din, tout, tin, 32, 1, nullptr);
  k_new_degree<<<grid, kThreads, 0, s>>>(src.xoff, dout, n, 32, (uint64_t)n + 1, dst.xoff);
  k_new_degree<<<grid, kThreads, 0, s>>>(src.xtoff, din, n, 32, (uint64_t)n + 1, dst.xtoff);
  if ((e = exclusive_scan_u32_ws(dst.xoff, n + 1, w.scan_off, s)) != cudaSuccess) return e;
  if ((e = exclusive_scan_u32_ws(dst.xtoff, n + 1, w.scan_off, s)) != cudaSuccess) return e;
  uint32_t *dbeg = w.ranges, *dend = dbeg + n, *ibeg = dend + n, *iend = ibeg + n;
  const uint32_t* keys[2][2] = {{du, iu}, {tdk, tik}};
  const uint32_t* vals[2][2] = {{dv, iv}, {tdv, tiv}};
  const uint32_t* ooff[2] = {src.xoff, src.xtoff};
  const uint32_t* oedg[2] = {src.xedg, src.xtedg};
  const uint32_t* nof[2] = {dst.xoff, dst.xtoff};
  uint32_t* ned[2] = {dst.xedg, dst.xtedg};
  const uint32_t* tch[2] = {tout, tin};
  for (int csr = 0; csr < 2; ++csr) {
    k_word_pop<<<grid, kThreads, 0, s>>>(tch[csr], words, w.cnt);
    if ((e = exclusive_scan_u32_ws(w.cnt, words + 1, w.scan_cnt, s)) != cudaSuccess) return e;
    k_touched_list<<<grid, kThreads, 0, s>>>(tch[csr], words, w.cnt, w.trow);
    if ((e = cudaMemsetAsync(w.ranges, 0, sizeof(uint32_t) * 4 * (size_t)n, s)) != cudaSuccess) return e;
    if (nd) k_batch_ranges<<<grid, kThreads, 0, s>>>(keys[csr][0], nd, dbeg, dend);
    if (ni) k_batch_ranges<<<grid, kThreads, 0, s>>>(keys[csr][1], ni, ibeg, iend);
    if ((e = cudaMemsetAsync(w.nbig, 0, 8, s)) != cudaSuccess) return e;
    const Runs r{ooff[csr], nof[csr], w.trow, 0, n, 0, w.cnt + words};
    k_copy_runs<<<grid, kThreads, 0, s>>>(r, oedg[csr], ned[csr]);
    k_merge_touched<<<grid, kThreads, 0, s>>>(r, oedg[csr], ned[csr], vals[csr][0], dbeg, dend, vals[csr][1], ibeg,
                                              iend, w.big, w.nbig);
    k_merge_big<<<grid, kThreads, 0, s>>>(r, oedg[csr], ned[csr], vals[csr][0], dbeg, dend, vals[csr][1], ibeg, iend,
                                          w.big, w.nbig);
  }
  k_out_degree<<<grid, kThreads, 0, s>>>(dst.xoff, 32, n, dst.xtdat);
  return cudaGetLastError();
}

// Ids below n and each list strictly ascending in (u, v): sets err bit 8 or 4
// otherwise.  The batch is read only if it passes (k_batch_check after it
// reads the rows of its ids).
__global__ void k_batch_valid(const uint32_t* b, uint32_t nd, uint32_t ni, uint32_t n, uint32_t* err) {
  const uint32_t *du = b, *dv = b + nd, *iu = b + 2 * (size_t)nd, *iv = iu + ni;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd + ni; i += gridDim.x * blockDim.x) {
    const bool del = i < nd;
    const uint32_t j = del ? i : i - nd;
    const uint32_t* u = del ? du : iu;
    const uint32_t* v = del ? dv : iv;
    if (u[j] >= n || v[j] >= n) atomicOr(err, 8u);
    else if (j > 0 && (u[j - 1] > u[j] || (u[j - 1] == u[j] && v[j - 1] >= v[j]))) atomicOr(err, 4u);
  }
}

__global__ void k_batch_check_if_valid(const uint32_t* __restrict__ off, const uint32_t* __restrict__ edg,
                                       const uint32_t* b, uint32_t nd, uint32_t ni, uint32_t* err) {
  if (*err) return;  // ids out of range or lists out of order: rows must not be read
  const uint32_t *du = b, *dv = b + nd, *iu = b + 2 * (size_t)nd, *iv = iu + ni;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd + ni; i += gridDim.x * blockDim.x) {
    const bool del = i < nd;
    const uint32_t u = del ? du[i] : iu[i - nd], v = del ? dv[i] : iv[i - nd];
    if (row_has(off, edg, nullptr, 32, u, v) != del) atomicOr(err, del ? 1u : 2u);
  }
}

void launch_batch_check(const uint32_t* xoff, const uint32_t* xedg, uint32_t n, const uint32_t* b, uint32_t nd,
                        uint32_t ni, uint32_t* err, int sms, cudaStream_t s) {
  if (nd + ni) {
    k_batch_valid<<<sms * 8, kThreads, 0, s>>>(b, nd, ni, n, err);
    k_batch_check_if_valid<<<sms * 8, kThreads, 0, s>>>(xoff, xedg, b, nd, ni, err);
  }
}

}  // namespace prx
