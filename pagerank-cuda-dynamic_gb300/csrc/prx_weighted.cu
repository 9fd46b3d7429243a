// prx_weighted.cu -- weighted PageRank and its adjoint.  No counterpart in
// the reference, whose graphs are unweighted (xtdat holds integer
// out-degrees, inc/pagerankCuda.hxx:87-109).
//
// Edge u -> v carries a weight w_uv > 0; rows are normalised,
// P_uv = w_uv / W_u with W_u = sum_v w_uv, and
//   forward:  r = (1 - alpha) t + alpha P^T r         (pull over in-edges)
//   adjoint:  lambda = alpha P lambda + g             (pull over out-edges)
// where g = dL/dr.  Both are Jacobi iterations of one pull kernel family,
// run on the in-CSR (forward) or on the out-CSR (adjoint, the reversed
// graph), stopped by the reference's L-inf test (:680,689).  With lambda and
// the converged r:
//   dL/dw_uv   = (r_u / W_u) (alpha lambda_v - lambda_u + g_u)
//   dL/dt      = (1 - alpha) lambda
//   dL/dalpha  = lambda . (P^T r - t)
// (dr = (I - alpha P^T)^-1 (alpha dP^T r + (P^T r - t) dalpha + (1-alpha) dt),
// and dP_uv'/dw_uv = (delta_vv' - P_uv') / W_u.)
//
// Rows go by length class: <= 64 one thread per row, <= 4096 one warp, else
// one block; every sum has a fixed order, so results are deterministic.
//
// Graphs with row segments (64-bit offsets, see GraphDev): px / pt are laid
// out like the edge arrays they follow (the same segment bases), and the
// weights and dL/dw stay in the compact out-CSR order a caller uses (edge j
// of a segment at its compact start + j).
#include <algorithm>
#include "prx_ctx.h"
#include "prx_device.cuh"

namespace prx {

void drop_weights(GraphDev& g) {
  cudaFree(g.px);
  cudaFree(g.pt);
  cudaFree(g.wsum);
  cudaFree(g.wseg);
  g.px = g.pt = g.wsum = nullptr;
  g.wseg = nullptr;
}

struct PullArgs {
  const uint32_t* off;            // rows to pull over
  const uint32_t* edg;
  const double* prob;             // P of each edge of the rows (laid out like edg)
  const unsigned long long* seg;  // row segments: the bases of edg and prob (null: one segment)
  uint32_t shift;
  const uint32_t* list;           // row ids by class
  uint32_t begin[NCLS + 1];
  const double* base;             // b_v, or base_const when null
  double base_scale;              // y_v = base_scale * b_v + alpha * sum
  double base_const;
  double alpha;
  const double* xin;              // null: the iterate of parity st->iter & 1
  double* x[2];
  double* y;                      // single sweep output (xin set)
  State* st;                      // null: single sweep, no L-inf
  uint32_t n;
};

__device__ __forceinline__ const double* pull_src(const PullArgs& a) {
  return a.xin ? a.xin : a.x[a.st->iter & 1];
}

__device__ __forceinline__ unsigned long long pull_finish(const PullArgs& a, uint32_t v, double sum) {
  const double b = a.base ? a.base[v] : a.base_const;
  const double y = fma(a.alpha, sum, a.base_scale * b);
  if (!a.st) {
    a.y[v] = y;
    return 0;
  }
  const int p = a.st->iter & 1;
  const double old = a.x[p][v];
  a.x[p ^ 1][v] = y;
  return dbits(fabs(y - old));
}

__global__ void __launch_bounds__(256) k_pull_low(PullArgs a) {
  if (a.st && a.st->done) return;
  const double* __restrict__ x = pull_src(a);
  unsigned long long emax = 0;
  for (uint32_t i = a.begin[LOW] + blockIdx.x * blockDim.x + threadIdx.x; i < a.begin[MID];
       i += gridDim.x * blockDim.x) {
    const uint32_t v = a.list[i];
    const uint64_t iv = seg_index(v, a.shift);
    const uint32_t s = a.off[iv], e = a.off[iv + 1];
    const uint64_t b = a.seg ? a.seg[(uint64_t)v >> a.shift] : 0;
    const uint32_t* __restrict__ edg = a.edg + b;
    const double* __restrict__ prob = a.prob + b;
    double acc = 0.0;
    uint32_t j = s;
    for (; j + 2 <= e; j += 2) {
      const uint32_t u0 = __ldg(edg + j), u1 = __ldg(edg + j + 1);
      const double p0 = __ldg(prob + j), p1 = __ldg(prob + j + 1);
      const double x0 = __ldg(x + u0), x1 = __ldg(x + u1);
      acc = fma(p0, x0, acc);
      acc = fma(p1, x1, acc);
    }
    if (j < e) acc = fma(__ldg(prob + j), __ldg(x + __ldg(edg + j)), acc);
    const unsigned long long d = pull_finish(a, v, acc);
    emax = d > emax ? d : emax;
  }
  if (a.st) block_max_bits(emax, &a.st->el_bits[a.st->iter & 1]);
}

__global__ void __launch_bounds__(256) k_pull_mid(PullArgs a) {
  if (a.st && a.st->done) return;
  const double* __restrict__ x = pull_src(a);
  const uint32_t lane = lane_id();
  unsigned long long emax = 0;
  for (uint32_t i = a.begin[MID] + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < a.begin[HIGH];
       i += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t v = a.list[i];
    const uint64_t iv = seg_index(v, a.shift);
    const uint32_t s = a.off[iv], e = a.off[iv + 1];
    const uint64_t b = a.seg ? a.seg[(uint64_t)v >> a.shift] : 0;
    const uint32_t* __restrict__ edg = a.edg + b;
    const double* __restrict__ prob = a.prob + b;
    double acc = 0.0;
    for (uint32_t j = s + lane; j < e; j += 32) acc = fma(__ldg(prob + j), __ldg(x + __ldg(edg + j)), acc);
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const unsigned long long d = pull_finish(a, v, acc);
      emax = d > emax ? d : emax;
    }
  }
  if (a.st) block_max_bits(emax, &a.st->el_bits[a.st->iter & 1]);
}

__global__ void __launch_bounds__(256) k_pull_high(PullArgs a) {
  __shared__ double part[8];
  if (a.st && a.st->done) return;
  const double* __restrict__ x = pull_src(a);
  unsigned long long emax = 0;
  for (uint32_t i = a.begin[HIGH] + blockIdx.x; i < a.begin[NCLS]; i += gridDim.x) {
    const uint32_t v = a.list[i];
    const uint64_t iv = seg_index(v, a.shift);
    const uint32_t s = a.off[iv], e = a.off[iv + 1];
    const uint64_t b = a.seg ? a.seg[(uint64_t)v >> a.shift] : 0;
    const uint32_t* __restrict__ edg = a.edg + b;
    const double* __restrict__ prob = a.prob + b;
    double acc = 0.0;
    for (uint32_t j = s + threadIdx.x; j < e; j += 256) acc = fma(__ldg(prob + j), __ldg(x + __ldg(edg + j)), acc);
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane_id() == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int k = 0; k < 8; ++k) t += part[k];
      const unsigned long long d = pull_finish(a, v, t);
      emax = d > emax ? d : emax;
    }
    __syncthreads();
  }
  if (a.st) block_max_bits(emax, &a.st->el_bits[a.st->iter & 1]);
}

__global__ void k_pull_fin(State* st) {
  if (st->done) return;
  const int p = st->iter & 1;
  const double el = __longlong_as_double((long long)st->el_bits[p]);
  st->last_delta = el;
  st->iter += 1;
  st->el_bits[p ^ 1] = 0;
  if (el < st->tol || st->iter >= st->max_iter) st->done = 1;
}

static int pull_grid(uint64_t work, int per_block, int cap) {
  const uint64_t b = (work + per_block - 1) / per_block;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(b, (uint64_t)cap));
}

static void pull_sweep(const PullArgs& a, int sms, cudaStream_t s, uint64_t& launches) {
  const uint32_t nl = a.begin[MID] - a.begin[LOW], nm = a.begin[HIGH] - a.begin[MID];
  const uint32_t nh = a.begin[NCLS] - a.begin[HIGH];
  if (nl) { k_pull_low<<<pull_grid(nl, 256, sms * 8), 256, 0, s>>>(a); ++launches; }
  if (nm) { k_pull_mid<<<pull_grid(nm, 8, sms * 8), 256, 0, s>>>(a); ++launches; }
  if (nh) { k_pull_high<<<pull_grid(nh, 1, sms * 4), 256, 0, s>>>(a); ++launches; }
}

// ---- weights ---------------------------------------------------------------------
// Warp per source u: W_u (lane-strided partial sums folded in lane order), px,
// and each out-edge's probability scattered to its in-CSR slot (binary search
// of u in v's ascending in-row).  err: 1 bad weight, 2 edge missing in xt.
// (Graph addressing of both CSRs: see the file comment; wseg: each out-CSR
// segment's compact start, null for one segment.)
struct WeightCsr {
  const uint32_t *xoff, *xedg, *xtoff, *xtedg;
  const unsigned long long *xbase, *xtbase, *wseg;
  uint32_t shift;
};

__global__ void __launch_bounds__(256) k_set_weights(WeightCsr c, const float* __restrict__ w, uint32_t n,
                                                     double* __restrict__ wsum, double* __restrict__ px,
                                                     double* __restrict__ pt, uint32_t* err) {
  const uint32_t lane = lane_id();
  for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += (gridDim.x * blockDim.x) >> 5) {
    const uint64_t iu = seg_index(u, c.shift);
    const uint32_t s = c.xoff[iu], e = c.xoff[iu + 1];
    const uint64_t bu = c.xbase ? c.xbase[(uint64_t)u >> c.shift] : 0;  // device position of the row's segment
    const uint64_t wu = c.wseg ? c.wseg[(uint64_t)u >> c.shift] : 0;    // its compact position
    double acc = 0.0;
    for (uint32_t j = s + lane; j < e; j += 32) {
      const float x = w[wu + j];
      if (!(x > 0.f) || !(x < INFINITY)) atomicOr(err, 1u);
      acc += (double)x;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) wsum[u] = acc;
    for (uint32_t j = s + lane; j < e; j += 32) {
      const double p = (double)w[wu + j] / acc;
      px[bu + j] = p;
      const uint32_t v = c.xedg[bu + j];
      const uint64_t iv = seg_index(v, c.shift);
      const uint64_t bv = c.xtbase ? c.xtbase[(uint64_t)v >> c.shift] : 0;
      const uint32_t* row = c.xtedg + bv;
      uint32_t lo = c.xtoff[iv], hi = c.xtoff[iv + 1];
      const uint32_t end = hi;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (row[mid] < u) lo = mid + 1;
        else hi = mid;
      }
      if (lo < end && row[lo] == u) pt[bv + lo] = p;
      else atomicOr(err, 2u);
    }
  }
}

// ---- gradients -------------------------------------------------------------------
// dL/dw_uv = (r_u / W_u) (alpha lambda_v - lambda_u + g_u), warp per source u.
__global__ void __launch_bounds__(256) k_grad_w(WeightCsr cs, const double* __restrict__ wsum,
                                                const double* __restrict__ r, const double* __restrict__ lam,
                                                const double* __restrict__ g, double alpha, uint32_t n,
                                                double* __restrict__ out) {
  const uint32_t lane = lane_id();
  for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += (gridDim.x * blockDim.x) >> 5) {
    const double f = r[u] / wsum[u], c = g[u] - lam[u];
    const uint64_t iu = seg_index(u, cs.shift);
    const uint64_t bu = cs.xbase ? cs.xbase[(uint64_t)u >> cs.shift] : 0;
    const uint64_t wu = cs.wseg ? cs.wseg[(uint64_t)u >> cs.shift] : 0;
    for (uint32_t j = cs.xoff[iu] + lane; j < cs.xoff[iu + 1]; j += 32)
      out[wu + j] = f * fma(alpha, lam[cs.xedg[bu + j]], c);
  }
}

__global__ void k_fill(double* __restrict__ x, double value, uint32_t n) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) x[v] = value;
}

__global__ void k_scale(const double* __restrict__ x, double f, uint32_t n, double* __restrict__ out) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) out[v] = f * x[v];
}

// Fixed-order dot product lambda . (y - t): per-block partial sums (grid-stride
// order, then the block tree), then one thread adds the partials in order.
__global__ void __launch_bounds__(256) k_dot_part(const double* __restrict__ lam, const double* __restrict__ y,
                                                  const double* __restrict__ t, double tconst, uint32_t n,
                                                  double* __restrict__ part) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    acc = fma(lam[v], y[v] - (t ? t[v] : tconst), acc);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_dot_final(const double* __restrict__ part, int np, double* __restrict__ out) {
  double acc = 0.0;
  for (int i = 0; i < np; ++i) acc += part[i];
  *out = acc;
}

}  // namespace prx

// ---- host side --------------------------------------------------------------------
static int wk_grow(prx_context* c, size_t doubles) {
  if (c->wk && c->wk_cap >= doubles) return PRX_OK;
  cudaFree(c->wk);
  c->wk = nullptr;
  c->wk_cap = 0;
  TRY_CUDA_ST(cudaMalloc(&c->wk, sizeof(double) * doubles));
  c->wk_cap = doubles;
  return PRX_OK;
}

static WeightCsr weight_csr(const GraphDev& g) {
  return WeightCsr{g.xoff, g.xedg, g.xtoff, g.xtedg, g.xbase, g.xtbase, g.wseg, g.seg_shift};
}

// Device slots of one CSR's edge array (its segments' positions and counts).
static uint64_t csr_slots(const GraphDev& g, const std::vector<uint64_t>& seg0, const std::vector<uint64_t>& pos) {
  if (g.nseg <= 1) return g.m ? g.m : 1;
  return pos.back() + (g.m - seg0.back()) + 4;
}

static PullArgs forward_args(const GraphDev& g, const double* t, double alpha) {
  PullArgs a{};
  a.off = g.xtoff;
  a.edg = g.xtedg;
  a.prob = g.pt;
  a.seg = g.xtbase;
  a.shift = g.seg_shift;
  a.list = g.cls_list;
  for (int k = 0; k <= NCLS; ++k) a.begin[k] = g.cls_begin[k];
  a.base = t;
  a.base_scale = 1.0 - alpha;
  a.base_const = 1.0 / (double)g.n;
  a.alpha = alpha;
  a.n = g.n;
  return a;
}

// Jacobi iterations of a from x[0] until the L-inf change is below tol or
// max_iter sweeps; returns the parity holding the answer.
static int pull_loop(prx_context* c, PullArgs& a, const prx_options& o, int* parity, prx_result* res) {
  cudaStream_t s = c->stream;
  a.st = c->st;
  a.xin = nullptr;
  launch_state_reset(c->st, o.max_iterations, o.tolerance, s);
  c->launches += 1;
  if (o.max_iterations > 0) {
    for (int k = 1;; k = std::min(2 * k, 16)) {
      for (int i = 0; i < k; ++i) {
        pull_sweep(a, c->sms, s, c->launches);
        k_pull_fin<<<1, 1, 0, s>>>(c->st);
        c->launches += 1;
      }
      TRY_CUDA_ST(cudaGetLastError());
      TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
      TRY_CUDA_ST(cudaStreamSynchronize(s));
      if (c->st_host[1].done) break;
    }
  } else {
    TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
    TRY_CUDA_ST(cudaStreamSynchronize(s));
  }
  *parity = c->st_host[1].iter & 1;
  if (res) {
    res->iterations += c->st_host[1].iter;
    res->last_delta = c->st_host[1].last_delta;
  }
  return PRX_OK;
}

static int weighted_check(prx_context* c, prx_graph* gr, const char* who) {
  if (!c || !gr || gr->ctx != c) {
    set_error(std::string(who) + ": bad context or graph");
    return PRX_EINVAL;
  }
  if (!gr->g.px) {
    set_error(std::string(who) + ": graph has no edge weights (prx_graph_set_weights)");
    return PRX_ESTATE;
  }
  return PRX_OK;
}

static void opts_or_default(const prx_options* o, prx_options* out) {
  if (o) *out = *o;
  else prx_options_default(out);
}

extern "C" {

int prx_graph_set_weights(prx_context* c, prx_graph* gr, const float* w) {
  if (!c || !gr || gr->ctx != c) FAIL(PRX_EINVAL, "prx_graph_set_weights: bad context or graph");
  GraphDev& g = gr->g;
  if (!g.xoff) FAIL(PRX_ESTATE, "prx_graph_set_weights: graph has no out-CSR");
  if (!w && g.m) FAIL(PRX_EINVAL, "prx_graph_set_weights: weights are NULL");
  TRY_CUDA_ST(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  drop_weights(g);
  TRY_CUDA_ST(cudaMalloc(&g.px, sizeof(double) * csr_slots(g, g.xseg0, g.xpos)));
  TRY_CUDA_ST(cudaMalloc(&g.pt, sizeof(double) * csr_slots(g, g.xtseg0, g.xtpos)));
  TRY_CUDA_ST(cudaMalloc(&g.wsum, sizeof(double) * (g.n ? g.n : 1)));
  if (g.nseg > 1) {  // each out-CSR segment's compact start
    TRY_CUDA_ST(cudaMalloc(&g.wseg, sizeof(unsigned long long) * g.nseg));
    TRY_CUDA_ST(cudaMemcpyAsync(g.wseg, g.xseg0.data(), sizeof(unsigned long long) * g.nseg,
                                cudaMemcpyHostToDevice, s));
  }
  if (!g.ocls_list) TRY_CUDA_ST(cudaMalloc(&g.ocls_list, sizeof(uint32_t) * (g.n ? g.n : 1)));
  launch_state_reset(c->st, 0, 0.0, s);
  if (g.n)
    k_set_weights<<<pull_grid((uint64_t)g.n * 32, 256, c->sms * 16), 256, 0, s>>>(weight_csr(g), w, g.n, g.wsum,
                                                                                  g.px, g.pt, &c->st->err);
  TRY_CUDA_ST(cudaGetLastError());
  const cudaError_t e = build_class_lists(g.xoff, g.seg_shift, g.n, g.mid_max, g.ocls_list, g.ocls_begin,
                                         g.ocls_edges, c->sms, s);
  TRY_CUDA_ST(e);
  TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
  TRY_CUDA_ST(cudaStreamSynchronize(s));
  const uint32_t err = c->st_host[1].err;
  if (err) {
    drop_weights(g);
    if (err & 1u) FAIL(PRX_EINVAL, "prx_graph_set_weights: every weight must be positive and finite");
    FAIL(PRX_EINVAL, "prx_graph_set_weights: an out-edge is missing from the in-CSR");
  }
  return PRX_OK;
}

int prx_solve_weighted(prx_context* c, prx_graph* gr, const double* t, const double* r0, const prx_options* opt,
                       double* r, prx_result* res) {
  int st = weighted_check(c, gr, "prx_solve_weighted");
  if (st) return st;
  prx_options o;
  opts_or_default(opt, &o);
  if (!(o.damping >= 0 && o.damping < 1)) FAIL(PRX_EINVAL, "prx_solve_weighted: damping must be in [0, 1)");
  const GraphDev& g = gr->g;
  prx_result rr{};
  if (g.n == 0) {
    if (res) *res = rr;
    return PRX_OK;
  }
  if (!r) FAIL(PRX_EINVAL, "prx_solve_weighted: r is NULL");
  TRY_CUDA_ST(cudaSetDevice(c->device));
  if ((st = wk_grow(c, 2 * (size_t)g.n))) return st;
  cudaStream_t s = c->stream;
  PullArgs a = forward_args(g, t, o.damping);
  a.x[0] = c->wk;
  a.x[1] = c->wk + g.n;
  const uint64_t l0 = c->launches;
  TRY_CUDA_ST(cudaEventRecord(c->ev[0], s));
  if (r0) {
    TRY_CUDA_ST(cudaMemcpyAsync(a.x[0], r0, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s));
  } else if (t) {
    TRY_CUDA_ST(cudaMemcpyAsync(a.x[0], t, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s));
  } else {
    k_fill<<<pull_grid(g.n, 256, c->sms * 16), 256, 0, s>>>(a.x[0], 1.0 / (double)g.n, g.n);
    c->launches += 1;
  }
  int parity = 0;
  if ((st = pull_loop(c, a, o, &parity, &rr))) return st;
  TRY_CUDA_ST(cudaMemcpyAsync(r, a.x[parity], sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s));
  TRY_CUDA_ST(cudaEventRecord(c->ev[1], s));
  TRY_CUDA_ST(cudaStreamSynchronize(s));
  float ms = 0;
  TRY_CUDA_ST(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  rr.time_ms = ms;
  rr.computation_time_ms = ms;
  rr.kernel_launches = c->launches - l0;
  if (res) *res = rr;
  return PRX_OK;
}

int prx_adjoint(prx_context* c, prx_graph* gr, const double* t, const double* r, const double* gl,
                const prx_options* opt, double* lambda, double* grad_w, double* grad_t, double* grad_alpha,
                prx_result* res) {
  int st = weighted_check(c, gr, "prx_adjoint");
  if (st) return st;
  prx_options o;
  opts_or_default(opt, &o);
  if (!(o.damping >= 0 && o.damping < 1)) FAIL(PRX_EINVAL, "prx_adjoint: damping must be in [0, 1)");
  const GraphDev& g = gr->g;
  prx_result rr{};
  if (g.n == 0) {
    if (grad_alpha) *grad_alpha = 0.0;
    if (res) *res = rr;
    return PRX_OK;
  }
  if (!r || !gl) FAIL(PRX_EINVAL, "prx_adjoint: r and g are required");
  TRY_CUDA_ST(cudaSetDevice(c->device));
  const int nparts = c->sms * 2;
  if ((st = wk_grow(c, 3 * (size_t)g.n + nparts + 1))) return st;
  cudaStream_t s = c->stream;
  const double alpha = o.damping;
  // lambda = alpha P lambda + g: the pull kernels on the out-CSR
  PullArgs a{};
  a.off = g.xoff;
  a.edg = g.xedg;
  a.prob = g.px;
  a.seg = g.xbase;
  a.shift = g.seg_shift;
  a.list = g.ocls_list;
  for (int k = 0; k <= NCLS; ++k) a.begin[k] = g.ocls_begin[k];
  a.base = gl;
  a.base_scale = 1.0;
  a.alpha = alpha;
  a.n = g.n;
  a.x[0] = c->wk;
  a.x[1] = c->wk + g.n;
  double* y = c->wk + 2 * (size_t)g.n;
  double* part = c->wk + 3 * (size_t)g.n;
  const uint64_t l0 = c->launches;
  TRY_CUDA_ST(cudaEventRecord(c->ev[0], s));
  TRY_CUDA_ST(cudaMemcpyAsync(a.x[0], gl, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s));
  int parity = 0;
  if ((st = pull_loop(c, a, o, &parity, &rr))) return st;
  const double* lam = a.x[parity];
  if (lambda) TRY_CUDA_ST(cudaMemcpyAsync(lambda, lam, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s));
  const int grid = pull_grid((uint64_t)g.n * 32, 256, c->sms * 16);
  if (grad_w) {
    k_grad_w<<<grid, 256, 0, s>>>(weight_csr(g), g.wsum, r, lam, gl, alpha, g.n, grad_w);
    c->launches += 1;
  }
  if (grad_t) {
    k_scale<<<pull_grid(g.n, 256, c->sms * 16), 256, 0, s>>>(lam, 1.0 - alpha, g.n, grad_t);
    c->launches += 1;
  }
  if (grad_alpha) {
    PullArgs f = forward_args(g, nullptr, 1.0);  // y = P^T r
    f.base_scale = 0.0;
    f.xin = r;
    f.y = y;
    f.st = nullptr;
    pull_sweep(f, c->sms, s, c->launches);
    k_dot_part<<<nparts, 256, 0, s>>>(lam, y, t, 1.0 / (double)g.n, g.n, part);
    k_dot_final<<<1, 1, 0, s>>>(part, nparts, part + nparts);
    c->launches += 2;
    TRY_CUDA_ST(cudaMemcpyAsync(grad_alpha, part + nparts, sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  TRY_CUDA_ST(cudaEventRecord(c->ev[1], s));
  TRY_CUDA_ST(cudaStreamSynchronize(s));
  TRY_CUDA_ST(cudaGetLastError());
  float ms = 0;
  TRY_CUDA_ST(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  rr.time_ms = ms;
  rr.computation_time_ms = ms;
  rr.kernel_launches = c->launches - l0;
  if (res) *res = rr;
  return PRX_OK;
}

}  // extern "C"
