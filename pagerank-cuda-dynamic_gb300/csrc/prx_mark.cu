// prx_mark.cu -- initial affected-vertex marking for DT / DF / DF-P.
//
// The reference keeps one byte flag per vertex and rescans all N flags in
// every marking kernel (inc/pagerankCuda.hxx:272-456).  Here the affected set
// is a bitmap (N/8 bytes, L2-resident at every graph size used), written with
// atomicOr; the rank-update kernels read it directly.  The resulting SET of
// affected vertices is the reference's:
//   seed:   deletion (u,v) -> expand u, mark v;  insertion (u,.) -> expand u
//           (pagerankAffectedFrontierPartialCukU :272-281)
//   expand: mark every out-neighbour of each vertex to expand
//           (pagerankAffectedExtend*CukU :313-366, pagerankAffectedFrontierCuW :405-412)
//   DT:     close the DF marking under out-edges (pagerankAffectedTraversalCuW
//           :438-456 repeats the expansion until the count stops growing; a
//           breadth-first closure over newly marked vertices gives the same set)
#include "prx_device.cuh"

namespace prx {

__device__ __forceinline__ void set_bit(uint32_t* bm, uint32_t v) {
  const uint32_t bit = 1u << (v & 31u);
  if (!(bm[v >> 5] & bit)) atomicOr(&bm[v >> 5], bit);
}

// Deletion (u,v): u queued for expansion, v affected.  Insertion (u,.): u
// queued.  The naff bitmap keeps each source once.
__global__ void k_mark_seed(SolveArgs a, const uint32_t* __restrict__ delu, const uint32_t* __restrict__ delv,
                            uint64_t nd, const uint32_t* __restrict__ insu, uint64_t ni) {
  State* st = a.st;
  uint32_t* b0 = a.bm[0];
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nd + ni;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t u = i < nd ? delu[i] : insu[i - nd];
    if (test_and_set(a.naff, u)) push(a.xl, &st->xcnt, u);
    if (i < nd) set_bit(b0, delv[i]);
  }
}

// Mark the out-neighbours of every queued source in bitmap 0, one warp per
// source; sources with more than 1024 out-edges go to the block-wide queue.
__global__ void __launch_bounds__(kThreads) k_expand_seeds(SolveArgs a) {
  const uint32_t count = a.st->xcnt;
  uint32_t* b0 = a.bm[0];
  const uint32_t lane = lane_id();
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < count; i += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t u = a.xl[i];
    const uint64_t iu = seg_index(u, a.seg_shift);
    const uint32_t b = a.xoff[iu], e = a.xoff[iu + 1];
    if (e - b > 1024) {
      if (lane == 0) push(a.xb, &a.st->xbcnt, u);
      continue;
    }
    const uint32_t* ed = seg_edges(a.xedg, a.xbase, a.seg_shift, u);
    for (uint32_t j = b + lane; j < e; j += 32) set_bit(b0, ed[j]);
  }
}

// DT: the closure starts from every vertex of the DF marking (naff <- vaff,
// :442).  Compact bitmap 0 into frontier 0.
__global__ void __launch_bounds__(kThreads) k_frontier_from_bitmap(SolveArgs a) {
  const uint32_t words = (a.n + 31) >> 5;
  const uint32_t lane = lane_id();
  const uint32_t* b0 = a.bm[0];
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += (gridDim.x * blockDim.x) >> 5) {
    if ((b0[w] >> lane) & 1u) push(a.fr[0], &a.st->fcnt[0], (w << 5) | lane);
  }
}

// DT closure without levels.  The closure is every vertex reachable from the
// DF marking (the reference grows it level by level until the count stops
// changing, :438-456; the order in which vertices are reached does not
// change the set), so persistent warps take reached vertices from a queue
// and mark their out-neighbours.
//   queue: frontier 0; its length is fcnt[0] (the tail), q_head counts items
//   taken, q_done items finished.  A slot is all ones until its producer has
//   written it (a consumer may take a slot the moment the tail covers it).
// A warp takes up to 32 items, one per lane.  A lane marks the out-neighbours
// of a vertex of out-degree <= 32 itself and goes on from one of the newly
// marked ones (up to kChain steps), so a long path -- the diameter of a road
// or grid graph -- is walked at one thread's memory latency per step rather
// than one queue round trip or one kernel launch per level.  The other new
// vertices wait in shared memory and reach the queue with one atomic per
// warp; vertices of larger out-degree are expanded by the whole warp.  Tail
// increments precede the warp's q_done increment (fence), so a warp that
// reads q_done and then the tail and finds them equal knows nothing is in
// flight: the closure is done.  Idle warps back off exponentially; every
// wait is bounded, and running out sets kErrClosureWait and returns.
constexpr uint32_t kQueueEmpty = 0xffffffffu;
constexpr int kClosureSpin = 1 << 20;
constexpr int kChain = 64;
constexpr int kQWarps = 4;           // warps per block of the queue kernel
constexpr uint32_t kQBuf = 2048;     // buffered new vertices per warp (32 KB of shared memory a block)

__global__ void __launch_bounds__(kQWarps * 32) k_closure_queue(SolveArgs a, uint32_t switch_at) {
  __shared__ uint32_t buf[kQWarps][kQBuf];
  __shared__ uint32_t nbuf[kQWarps];
  State* st = a.st;
  volatile uint32_t* vhead = &st->q_head;
  volatile uint32_t* vtail = &st->fcnt[0];
  volatile uint32_t* vdone = &st->q_done;
  volatile uint32_t* verr = &st->err;
  uint32_t* queue = a.fr[0];
  volatile const uint32_t* vq = queue;
  uint32_t* reached = a.bm[0];
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  auto flush = [&]() {  // the warp's buffered vertices to the queue
    __syncwarp();
    const uint32_t k = nbuf[w];
    uint32_t base = 0;
    if (lane == 0 && k) base = atomicAdd(&st->fcnt[0], k);
    base = __shfl_sync(0xffffffffu, base, 0);
    for (uint32_t i = lane; i < k; i += 32) queue[base + i] = buf[w][i];
    __syncwarp();
    if (lane == 0) nbuf[w] = 0;
    __syncwarp();
  };
  if (lane == 0) nbuf[w] = 0;
  __syncwarp();
  for (;;) {
    uint32_t h = 0, cnt = 0;
    if (lane == 0) {
      unsigned backoff = 64;
      for (int spin = 0;;) {
        if (*verr) break;
        const uint32_t head = *vhead;
        const uint32_t done = *vdone;
        __threadfence();
        const uint32_t tail = *vtail;
        if (tail > switch_at && tail / 8u > done) break;  // exploding: pull rounds finish it
        if (head < tail) {
          const uint32_t take = min(32u, tail - head);
          if (atomicCAS(&st->q_head, head, head + take) == head) {
            h = head;
            cnt = take;
            break;
          }
          continue;
        }
        if (done == tail) break;  // closed
        if (++spin > kClosureSpin) {
          atomicOr(&st->err, kErrClosureWait);
          break;
        }
        __nanosleep(backoff);
        backoff = min(backoff * 2, 8192u);
      }
    }
    h = __shfl_sync(0xffffffffu, h, 0);
    cnt = __shfl_sync(0xffffffffu, cnt, 0);
    if (cnt == 0) break;
    uint32_t u = kQueueEmpty;
    if (lane < cnt) {
      for (int spin = 0; (u = vq[h + lane]) == kQueueEmpty;) {
        if (++spin > kClosureSpin || *verr) {
          atomicOr(&st->err, kErrClosureWait);
          break;
        }
        __nanosleep(64);
      }
    }
    for (int step = 0; step < kChain; ++step) {
      const bool valid = u != kQueueEmpty;
      if (!__any_sync(0xffffffffu, valid)) break;
      uint32_t b = 0, e = 0;
      if (valid) {
        const uint64_t iu = seg_index(u, a.seg_shift);
        b = a.xoff[iu];
        e = a.xoff[iu + 1];
      }
      const bool small = e - b <= 32u;
      uint32_t next = kQueueEmpty;
      if (valid && small) {
        const uint32_t* ed = seg_edges(a.xedg, a.xbase, a.seg_shift, u);
        for (uint32_t j = b; j < e; ++j) {
          const uint32_t x = ed[j];
          if (test_and_set(reached, x)) {
            if (next == kQueueEmpty) next = x;  // this lane goes on from x
            else buf[w][atomicAdd(&nbuf[w], 1u)] = x;
          }
        }
      }
      unsigned big = __ballot_sync(0xffffffffu, valid && !small);
      while (big) {
        const int src = __ffs(big) - 1;
        big &= big - 1;
        const uint32_t ub = __shfl_sync(0xffffffffu, u, src);
        const uint32_t bb = __shfl_sync(0xffffffffu, b, src), eb = __shfl_sync(0xffffffffu, e, src);
        const uint32_t* ed = seg_edges(a.xedg, a.xbase, a.seg_shift, ub);
        for (uint32_t j = bb + lane; j < eb; j += 32) {
          const uint32_t x = ed[j];
          if (test_and_set(reached, x)) push(queue, &st->fcnt[0], x);
        }
      }
      u = next;
      __syncwarp();
      if (nbuf[w] > kQBuf - 32u * 32u) flush();  // room for one more step of every lane
    }
    if (u != kQueueEmpty) buf[w][atomicAdd(&nbuf[w], 1u)] = u;  // chain cut: back to the queue
    flush();
    __threadfence();  // this warp's tail increments and slots before its q_done increment
    __syncwarp();
    if (lane == 0) atomicAdd(&st->q_done, cnt);
  }
}

// Closure round r by pulling (the reached set is bitmap 0; set semantics, so
// the order rounds and warps add vertices in does not matter).  Round r adds
// to pcnt[r % 3] and zeroes pcnt[(r+1) % 3], which round r-2 filled and round
// r-1 read.  A round after one that added nothing sets pdone and returns, and
// so does every round after it.  A warp is the only writer of its bitmap
// word here; other warps may read it while it changes, and a bit seen set
// early only speeds the closure up.
__global__ void __launch_bounds__(kThreads) k_closure_pull(SolveArgs a, uint32_t round) {
  State* st = a.st;
  if (st->pdone) return;
  if (round > 0 && st->pcnt[(round - 1) % 3] == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->pdone = 1;
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) st->pcnt[(round + 1) % 3] = 0;
  uint32_t* reached = a.bm[0];
  const uint32_t words = (a.n + 31) >> 5;
  const uint32_t lane = lane_id();
  unsigned long long added = 0;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t word = reached[w];
    if (word == 0xffffffffu) continue;
    const uint32_t v = (w << 5) | lane;
    bool hit = false;
    if (v < a.n && !((word >> lane) & 1u)) {
      const uint64_t iv = seg_index(v, a.seg_shift);
      const uint32_t e = a.xtoff[iv + 1];
      const uint32_t* ed = seg_edges(a.xtedg, a.xtbase, a.seg_shift, v);
      for (uint32_t j = a.xtoff[iv]; j < e && !hit; ++j) {
        const uint32_t u = ed[j];
        hit = (reached[u >> 5] >> (u & 31u)) & 1u;
      }
    }
    const unsigned add = __ballot_sync(0xffffffffu, hit);
    if (lane == 0 && add) {
      reached[w] = word | add;
      added += __popc(add);
    }
  }
  unsigned long long total = added;  // block sum, then one atomic per block
  for (int o = 16; o; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
  __shared__ unsigned long long part[kThreads / 32];
  if (lane == 0) part[threadIdx.x >> 5] = total;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = 0;
    for (int k = 0; k < kThreads / 32; ++k) b += part[k];
    if (b) atomicAdd(&st->pcnt[round % 3], (uint32_t)b);
  }
}

__global__ void k_popcount(const uint32_t* __restrict__ bm, uint32_t words, unsigned long long* out) {
  unsigned long long x = 0;
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += gridDim.x * blockDim.x) x += __popc(bm[w]);
  block_sum_u64(x, out);
}

__global__ void k_flags_from_bitmap(const uint32_t* __restrict__ bm, uint8_t* __restrict__ out, uint32_t n) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    out[v] = (bm[v >> 5] >> (v & 31)) & 1u;
}

__global__ void k_state_reset(State* st, int max_iter, double tol) {
  st->el_bits[0] = st->el_bits[1] = 0;
  st->iter = 0;
  st->done = max_iter <= 0;  // while (l < L) runs no sweep when L <= 0
  st->max_iter = max_iter;
  st->tol = tol;
  st->last_delta = 0;
  for (int p = 0; p < 2; ++p)
    for (int c = 0; c < NCLS; ++c) st->cnt[p][c] = 0;
  st->xcnt = 0;
  st->fcnt[0] = st->fcnt[1] = st->fcnt[2] = 0;
  st->pcnt[0] = st->pcnt[1] = st->pcnt[2] = 0;
  st->pdone = 0;
  st->err = 0;
  st->edges = 0;
  st->affected = 0;
  st->nfcnt = 0;
  st->xbcnt = 0;
  st->k32 = 0;
  st->inner_done = 0;
  st->rounds = 0;
  st->el32_bits[0] = st->el32_bits[1] = 0;
  st->e32max_bits[0] = st->e32max_bits[1] = 0;
  st->graph_rounds = 0;
  st->graph_inner = 0;
  st->q_head = 0;
  st->q_done = 0;
  st->el32_prev[0] = st->el32_prev[1] = 0;
}

// ---- launchers ------------------------------------------------------------------
void launch_mark_seed(const SolveArgs& a, const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                      const uint32_t* insu, uint64_t ni, int sms, cudaStream_t s) {
  const uint64_t want = (nd + ni + kThreads - 1) / kThreads;
  const int grid = (int)(want < (uint64_t)sms * 8 ? (want ? want : 1) : (uint64_t)sms * 8);
  k_mark_seed<<<grid, kThreads, 0, s>>>(a, delu, delv, nd, insu, ni);
}

void launch_expand_seeds(const SolveArgs& a, int sms, cudaStream_t s) {
  k_expand_seeds<<<sms * 4, kThreads, 0, s>>>(a);
}

void launch_frontier_from_bitmap(const SolveArgs& a, int sms, cudaStream_t s) {
  k_frontier_from_bitmap<<<sms * 4, kThreads, 0, s>>>(a);
}

void launch_closure_queue(const SolveArgs& a, uint32_t switch_at, int sms, cudaStream_t s) {
  k_closure_queue<<<sms * 2, kQWarps * 32, 0, s>>>(a, switch_at);
}

void launch_closure_pull(const SolveArgs& a, uint32_t round, int sms, cudaStream_t s) {
  k_closure_pull<<<sms * 8, kThreads, 0, s>>>(a, round);
}

void launch_popcount(const uint32_t* bm, uint32_t n, unsigned long long* out, int sms, cudaStream_t s) {
  k_popcount<<<sms * 2, kThreads, 0, s>>>(bm, (n + 31) / 32, out);
}

void launch_flags_from_bitmap(const uint32_t* bm, uint8_t* out, uint32_t n, cudaStream_t s) {
  const uint32_t grid = (n + kThreads - 1) / kThreads;
  k_flags_from_bitmap<<<grid < 4096 ? (grid ? grid : 1) : 4096, kThreads, 0, s>>>(bm, out, n);
}

void launch_state_reset(State* st, int max_iter, double tol, cudaStream_t s) {
  k_state_reset<<<1, 1, 0, s>>>(st, max_iter, tol);
}

}  // namespace prx
