// prx_batch.cu -- apply a tidied batch update to the device CSRs.
//
// The reference applies a batch on the host, vertex by vertex
// (applyBatchUpdateOmpU, inc/batch.hxx:239-247), and rebuilds the transpose
// from scratch (transposeWithDegreeOmp, inc/transpose.hxx:128-134); both are
// outside its timed region.  Here the update runs on the device:
//   1. check the batch is tidy against the current graph (deletions exist,
//      insertions do not), so the merge below cannot go wrong;
//   2. per-vertex degree deltas and "touched" bitmaps for both CSRs;
//   3. new offsets = exclusive scan of the new degrees;
//   4. one warp per row: untouched rows are copied (coalesced), touched rows
//      are merged (old row minus deletions, plus insertions, ascending -- the
//      LazyBitset order the reference keeps);
//   5. out-degrees and the in-degree classes are refreshed.
// The in-CSR needs the batch ordered by (v, u); the host prepares that order.
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

__device__ __forceinline__ bool row_has(const uint32_t* off, const uint32_t* edg, uint32_t u, uint32_t v) {
  const uint32_t b = off[u], len = off[u + 1] - b;
  const uint32_t i = lower_bound_u32(edg + b, len, v);
  return i < len && edg[b + i] == v;
}

// Flags err if a deletion is missing or an insertion already exists.
__global__ void k_batch_check(const uint32_t* __restrict__ off, const uint32_t* __restrict__ edg,
                              const uint32_t* du, const uint32_t* dv, uint32_t nd,
                              const uint32_t* iu, const uint32_t* iv, uint32_t ni, uint32_t* err) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd + ni; i += gridDim.x * blockDim.x) {
    const bool del = i < nd;
    const uint32_t u = del ? du[i] : iu[i - nd], v = del ? dv[i] : iv[i - nd];
    if (row_has(off, edg, u, v) != del) atomicOr(err, del ? 1u : 2u);
  }
}

__global__ void k_batch_deltas(const uint32_t* du, const uint32_t* dv, uint32_t nd,
                               const uint32_t* iu, const uint32_t* iv, uint32_t ni,
                               int32_t* dout, int32_t* din, uint32_t* tout, uint32_t* tin) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd + ni; i += gridDim.x * blockDim.x) {
    const bool del = i < nd;
    const uint32_t u = del ? du[i] : iu[i - nd], v = del ? dv[i] : iv[i - nd];
    atomicAdd(dout + u, del ? -1 : 1);
    atomicAdd(din + v, del ? -1 : 1);
    atomicOr(tout + (u >> 5), 1u << (u & 31));
    atomicOr(tin + (v >> 5), 1u << (v & 31));
  }
}

// deg[v] = old degree + delta (v < n); deg[n] = 0, so the exclusive scan
// leaves the edge count in deg[n].
__global__ void k_new_degree(const uint32_t* __restrict__ off, const int32_t* __restrict__ delta, uint32_t n,
                             uint32_t* __restrict__ deg) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x)
    deg[v] = v < n ? (uint32_t)((int64_t)(off[v + 1] - off[v]) + delta[v]) : 0u;
}

// Rows keyed by `key` (u for the out-CSR, v for the in-CSR); deletions and
// insertions sorted by (key, val).  A warp per group of 32 rows.
//
// Untouched rows keep their ids; their old edges lie in one contiguous range
// with the touched rows' edges in between.  The warp walks the group's whole
// old range 32 positions at a time (coalesced); each lane finds the row of
// its position by a binary search over the 32 row starts (held one per lane,
// read with shuffles) and, if that row is untouched, copies the id to the
// row's new start plus its offset in the row.
//
// A touched row is merged by ranks, 32 elements at a time: a kept old id w
// goes to (its index) - (deleted ids before it) + (inserted ids below w); an
// inserted id x goes to (its index among the row's insertions) + (old ids
// below x) - (deleted ids below x).  The batch is tidy (deletions are old
// ids, insertions are not), so these are the positions of the sorted merge;
// every lane finds its own with binary searches, and hub rows with 100k ids
// take no serial pass.
__device__ void merge_row(const uint32_t* __restrict__ oedg, uint32_t* __restrict__ nedg, uint32_t os, uint32_t len,
                          uint32_t ns, const uint32_t* dv, uint32_t d0, uint32_t d1, const uint32_t* iv, uint32_t i0,
                          uint32_t i1, uint32_t lane) {
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t* rdel = dv + d0;
  const uint32_t* rins = iv + i0;
  const uint32_t nrd = d1 - d0, nri = i1 - i0;
  uint32_t deleted = 0;  // deleted old ids in the chunks before this one
  for (uint32_t base = 0; base < len; base += 32) {
    const uint32_t j = base + lane;
    const bool valid = j < len;
    const uint32_t w = valid ? oedg[os + j] : 0u;
    const uint32_t p = valid ? lower_bound_u32(rdel, nrd, w) : 0u;
    const bool del = valid && p < nrd && rdel[p] == w;
    const unsigned dmask = __ballot_sync(0xffffffffu, del);
    if (valid && !del) nedg[ns + j - (deleted + __popc(dmask & lt)) + lower_bound_u32(rins, nri, w)] = w;
    deleted += __popc(dmask);
  }
  for (uint32_t k = lane; k < nri; k += 32) {
    const uint32_t x = rins[k];
    nedg[ns + k + lower_bound_u32(oedg + os, len, x) - lower_bound_u32(rdel, nrd, x)] = x;
  }
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

__global__ void __launch_bounds__(kThreads) k_merge_rows(const uint32_t* __restrict__ ooff, const uint32_t* __restrict__ oedg,
                                                         const uint32_t* __restrict__ noff, uint32_t* __restrict__ nedg, uint32_t n,
                                                         const uint32_t* dv, const uint32_t* __restrict__ dbeg,
                                                         const uint32_t* __restrict__ dend, const uint32_t* iv,
                                                         const uint32_t* __restrict__ ibeg, const uint32_t* __restrict__ iend,
                                                         const uint32_t* __restrict__ touched) {
  const uint32_t lane = lane_id();
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t groups = (n + 31) >> 5;
  for (uint32_t gi = warp; gi < groups; gi += nwarps) {
    const uint32_t r0 = gi << 5;
    const uint32_t cnt = min(32u, n - r0);           // rows in this group
    const uint32_t rl = r0 + min(lane, cnt - 1);     // lanes past the end repeat the last row
    const uint32_t os = ooff[rl], ns = noff[rl];
    const uint32_t oend = ooff[r0 + cnt];
    const uint32_t tw = touched[gi];
    const uint32_t o0 = __shfl_sync(0xffffffffu, os, 0);
    for (uint32_t pb = o0; pb < oend; pb += 128) {  // 4 positions per lane in flight
      uint32_t val[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t p = pb + 32u * q + lane;
        val[q] = p < oend ? oedg[p] : 0u;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t p = pb + 32u * q + lane;
        // the row of position p: the last of the group's rows starting at or before p
        uint32_t i = 0;
#pragma unroll
        for (uint32_t step = 16; step; step >>= 1) {
          const uint32_t c = i + step;
          const uint32_t sc = __shfl_sync(0xffffffffu, os, c < cnt ? c : cnt - 1);
          if (c < cnt && sc <= p) i = c;
        }
        const uint32_t si = __shfl_sync(0xffffffffu, os, i), ni_ = __shfl_sync(0xffffffffu, ns, i);
        if (p < oend && !((tw >> i) & 1u)) nedg[ni_ + (p - si)] = val[q];
      }
    }
    for (uint32_t m = tw; m; m &= m - 1) {           // touched rows, one at a time with the whole warp
      const uint32_t i = __ffs(m) - 1;
      const uint32_t r = r0 + i;
      const uint32_t s = ooff[r], e = ooff[r + 1];
      merge_row(oedg, nedg, s, e - s, noff[r], dv, dbeg[r], dend[r], iv, ibeg[r], iend[r], lane);
    }
  }
}

__global__ void k_out_degree(const uint32_t* __restrict__ off, uint32_t n, uint32_t* __restrict__ deg) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    deg[v] = off[v + 1] - off[v];
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

// b: device array [du | dv | iu | iv | tdk | tdv | tik | tiv] where the t*
// arrays are the batch sorted by (v, u).  Returns cudaErrorInvalidValue if the
// batch is not tidy for the current graph (nothing is modified then).
cudaError_t apply_batch_device(GraphDev& g, const uint32_t* b, uint64_t nd64, uint64_t ni64,
                               int sms, cudaStream_t s) {
  cudaError_t err = cudaSuccess;
  const uint32_t n = g.n, nd = (uint32_t)nd64, ni = (uint32_t)ni64;
  const uint32_t *du = b, *dv = b + nd, *iu = b + 2 * (size_t)nd, *iv = iu + ni;
  const uint32_t *tdk = iv + ni, *tdv = tdk + nd, *tik = tdv + nd, *tiv = tik + ni;
  const uint64_t m2 = g.m - nd + ni;
  const uint32_t words = (n + 31) / 32;
  const int grid = sms * 8;
  uint32_t *scratch = nullptr, *noff = nullptr, *ntoff = nullptr, *nedg = nullptr, *ntedg = nullptr, *ndat = nullptr;
  uint32_t* ranges = nullptr;
  int32_t *dout, *din;
  uint32_t *tout, *tin, *flag;
  uint32_t hflag = 0;
  // scratch: deltas (2n) + touched (2 words) + flag
  PRX_CU(graph_alloc(&scratch, sizeof(uint32_t) * (2 * (size_t)n + 2 * (size_t)words + 1), s));
  dout = (int32_t*)scratch; din = dout + n;
  tout = (uint32_t*)(din + n); tin = tout + words; flag = tin + words;
  PRX_CU(cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * (2 * (size_t)n + 2 * (size_t)words + 1), s));
  if (nd + ni) {
    k_batch_check<<<grid, kThreads, 0, s>>>(g.xoff, g.xedg, du, dv, nd, iu, iv, ni, flag);
    PRX_CU(cudaMemcpyAsync(&hflag, flag, 4, cudaMemcpyDeviceToHost, s));
    PRX_CU(cudaStreamSynchronize(s));
    if (hflag) { err = cudaErrorInvalidValue; goto done; }
    k_batch_deltas<<<grid, kThreads, 0, s>>>(du, dv, nd, iu, iv, ni, dout, din, tout, tin);
  }
  PRX_CU(graph_alloc(&noff, sizeof(uint32_t) * ((size_t)n + 1), s));
  PRX_CU(graph_alloc(&ntoff, sizeof(uint32_t) * ((size_t)n + 1), s));
  PRX_CU(graph_alloc(&nedg, sizeof(uint32_t) * (m2 ? m2 : 1), s));
  PRX_CU(graph_alloc(&ntedg, sizeof(uint32_t) * edge_slots(m2), s));
  PRX_CU(graph_alloc(&ndat, sizeof(uint32_t) * (n ? n : 1), s));
  k_new_degree<<<grid, kThreads, 0, s>>>(g.xoff, dout, n, noff);
  k_new_degree<<<grid, kThreads, 0, s>>>(g.xtoff, din, n, ntoff);
  PRX_CU(exclusive_scan_u32(noff, n + 1, s));
  PRX_CU(exclusive_scan_u32(ntoff, n + 1, s));
  // each CSR: the per-row ranges of its deletions and insertions, then the merge
  PRX_CU(graph_alloc(&ranges, sizeof(uint32_t) * 4 * (size_t)(n ? n : 1), s));
  {
    uint32_t *dbeg = ranges, *dend = dbeg + n, *ibeg = dend + n, *iend = ibeg + n;
    const uint32_t* keys[2][2] = {{du, iu}, {tdk, tik}};
    const uint32_t* vals[2][2] = {{dv, iv}, {tdv, tiv}};
    for (int csr = 0; csr < 2; ++csr) {
      PRX_CU(cudaMemsetAsync(ranges, 0, sizeof(uint32_t) * 4 * (size_t)n, s));
      if (nd) k_batch_ranges<<<grid, kThreads, 0, s>>>(keys[csr][0], nd, dbeg, dend);
      if (ni) k_batch_ranges<<<grid, kThreads, 0, s>>>(keys[csr][1], ni, ibeg, iend);
      if (csr == 0)
        k_merge_rows<<<grid, kThreads, 0, s>>>(g.xoff, g.xedg, noff, nedg, n, vals[0][0], dbeg, dend, vals[0][1],
                                               ibeg, iend, tout);
      else
        k_merge_rows<<<grid, kThreads, 0, s>>>(g.xtoff, g.xtedg, ntoff, ntedg, n, vals[1][0], dbeg, dend, vals[1][1],
                                               ibeg, iend, tin);
    }
  }
  k_out_degree<<<grid, kThreads, 0, s>>>(noff, n, ndat);
  PRX_CU(cudaGetLastError());
  PRX_CU(cudaStreamSynchronize(s));
  graph_free({g.xoff, g.xedg, g.xtoff, g.xtedg, g.xtdat});
  g.xoff = noff; g.xedg = nedg; g.xtoff = ntoff; g.xtedg = ntedg; g.xtdat = ndat;
  noff = nedg = ntoff = ntedg = ndat = nullptr;
  g.m = m2;
  g.m_cap = m2;
  PRX_CU(build_classes(g, sms, s));
done:
  if (scratch) cudaFreeAsync(scratch, s);
  if (ranges) cudaFreeAsync(ranges, s);
  graph_free({noff, ntoff, nedg, ntedg, ndat});
  return err;
}

}  // namespace prx
