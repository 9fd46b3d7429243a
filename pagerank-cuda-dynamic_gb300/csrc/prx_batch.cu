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
// insertions sorted by (key, val).
__global__ void __launch_bounds__(kThreads) k_merge_rows(const uint32_t* __restrict__ ooff, const uint32_t* __restrict__ oedg,
                                                         const uint32_t* __restrict__ noff, uint32_t* __restrict__ nedg, uint32_t n,
                                                         const uint32_t* dk, const uint32_t* dv, uint32_t nd,
                                                         const uint32_t* ik, const uint32_t* iv, uint32_t ni,
                                                         const uint32_t* __restrict__ touched) {
  const uint32_t lane = lane_id();
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t r = warp; r < n; r += nwarps) {
    const uint32_t os = ooff[r], oe = ooff[r + 1], ns = noff[r];
    if (!((touched[r >> 5] >> (r & 31)) & 1u)) {
      for (uint32_t j = lane; j < oe - os; j += 32) nedg[ns + j] = oedg[os + j];
      continue;
    }
    if (lane != 0) continue;
    uint32_t di = lower_bound_u32(dk, nd, r), ii = lower_bound_u32(ik, ni, r), i = os, k = ns;
    for (;;) {
      const bool has_old = i < oe;
      const bool has_ins = ii < ni && ik[ii] == r;
      if (!has_old && !has_ins) break;
      if (has_old && (!has_ins || oedg[i] < iv[ii])) {
        const uint32_t w = oedg[i++];
        while (di < nd && dk[di] == r && dv[di] < w) ++di;
        if (di < nd && dk[di] == r && dv[di] == w) { ++di; continue; }
        nedg[k++] = w;
      } else {
        nedg[k++] = iv[ii++];
      }
    }
  }
}

__global__ void k_out_degree(const uint32_t* __restrict__ off, uint32_t n, uint32_t* __restrict__ deg) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    deg[v] = off[v + 1] - off[v];
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
  int32_t *dout, *din;
  uint32_t *tout, *tin, *flag;
  uint32_t hflag = 0;
  // scratch: deltas (2n) + touched (2 words) + flag
  PRX_CU(cudaMallocAsync(&scratch, sizeof(uint32_t) * (2 * (size_t)n + 2 * (size_t)words + 1), s));
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
  k_merge_rows<<<grid, kThreads, 0, s>>>(g.xoff, g.xedg, noff, nedg, n, du, dv, nd, iu, iv, ni, tout);
  k_merge_rows<<<grid, kThreads, 0, s>>>(g.xtoff, g.xtedg, ntoff, ntedg, n, tdk, tdv, nd, tik, tiv, ni, tin);
  k_out_degree<<<grid, kThreads, 0, s>>>(noff, n, ndat);
  PRX_CU(cudaGetLastError());
  PRX_CU(cudaStreamSynchronize(s));
  cudaFree(g.xoff); cudaFree(g.xedg); cudaFree(g.xtoff); cudaFree(g.xtedg); cudaFree(g.xtdat);
  g.xoff = noff; g.xedg = nedg; g.xtoff = ntoff; g.xtedg = ntedg; g.xtdat = ndat;
  noff = nedg = ntoff = ntedg = ndat = nullptr;
  g.m = m2;
  g.m_cap = m2;
  PRX_CU(build_classes(g, sms, s));
done:
  if (scratch) cudaFreeAsync(scratch, s);
  if (noff) cudaFree(noff);
  if (ntoff) cudaFree(ntoff);
  if (nedg) cudaFree(nedg);
  if (ntedg) cudaFree(ntedg);
  if (ndat) cudaFree(ndat);
  return err;
}

}  // namespace prx
