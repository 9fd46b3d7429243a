// prx_api.cu -- the C ABI (include/pagerank_gb300.h): contexts, device graphs
// and the solve driver that replaces pagerankInvokeCuda + pagerankLoopCuU
// (inc/pagerankCuda.hxx:675-849).
//
// Differences from the reference's driver, none of which changes a result:
//  - the graph stays on the device across solves (the reference re-uploads
//    and re-partitions it on every call, :777-813);
//  - the loop keeps its state on the device (iteration count, L-inf delta,
//    done flag) and the host reads it back once per batch of iterations
//    instead of after each one (:685), or never (CUDA-graph loop);
//  - errors come back as status codes instead of exit() (inc/_cuda.hxx:136).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>
#include "prx_ctx.h"

using namespace prx;

namespace prx {
static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
}  // namespace prx

extern "C" {

void prx_options_default(prx_options* o) {
  if (!o) return;
  o->repeat = 1;
  o->tolerance = 1e-10;
  o->frontier_tolerance = 1e-6;
  o->prune_tolerance = 1e-6;
  o->damping = 0.85;
  o->max_iterations = 500;
  o->precision = PRX_FP64;
  o->loop = PRX_LOOP_AUTO;
  o->partition = 0;
  o->timing = 0;
  o->expansion = 0;
  o->chunk_vertices = 0;
  o->refine_sweeps = 0;
  o->l2_fetch_bytes = 0;
  o->require_convergence = 0;
  o->hot_sources = 0;
  o->int_adds = 0;
}

const char* prx_status_string(int s) {
  switch (s) {
    case PRX_OK: return "ok";
    case PRX_EINVAL: return "invalid argument";
    case PRX_ENOMEM: return "out of memory";
    case PRX_ECUDA: return "CUDA error";
    case PRX_ETIMEOUT: return "device wait timed out";
    case PRX_ERANGE: return "size out of range";
    case PRX_ESTATE: return "invalid state";
    case PRX_ENOCONV: return "did not converge";
    default: return "unknown status";
  }
}

const char* prx_last_error(void) { return g_last_error.c_str(); }

int prx_context_create(int device, prx_context** out) {
  if (!out) FAIL(PRX_EINVAL, "prx_context_create: out is NULL");
  *out = nullptr;
  int count = 0;
  TRY_CUDA_ST(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) FAIL(PRX_EINVAL, "prx_context_create: no such device");
  TRY_CUDA_ST(cudaSetDevice(device));
  prx_context* c = new prx_context();
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->st, sizeof(State));
  if (e == cudaSuccess) e = cudaMallocHost(&c->st_host, 2 * sizeof(State));
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
  if (e != cudaSuccess) {
    set_error(std::string("prx_context_create: ") + cudaGetErrorString(e));
    prx_context_destroy(c);
    return e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
  }
  *out = c;
  return PRX_OK;
}

static void free_ws(prx_context* c) {
  for (int p = 0; p < 2; ++p) {
    cudaFree(c->r[p]); c->r[p] = nullptr;
    cudaFree(c->c[p]); c->c[p] = nullptr;
    for (int k = 0; k < NCLS; ++k) { cudaFree(c->lists[p][k]); c->lists[p][k] = nullptr; }
  }
  for (auto& f : c->fr) { cudaFree(f); f = nullptr; }
  cudaFree(c->acc64); c->acc64 = nullptr;
  cudaFree(c->acc32); c->acc32 = nullptr;
  for (auto& h : c->ch) { cudaFree(h); h = nullptr; }
  c->ch_n = 0;
  cudaFree(c->flags); c->flags = nullptr;
  for (auto& b : c->bm) { cudaFree(b); b = nullptr; }
  for (auto& b : c->nf) { cudaFree(b); b = nullptr; }
  cudaFree(c->xb); c->xb = nullptr;
  cudaFree(c->naff); c->naff = nullptr;
  cudaFree(c->ever); c->ever = nullptr;
  cudaFree(c->pf); c->pf = nullptr;
  cudaFree(c->xl); c->xl = nullptr;
  c->ws_n = 0;
  c->ws_dyn = false;
}

int prx_context_destroy(prx_context* c) {
  if (!c) return PRX_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_ws(c);
  ppr_free(c->ppr);
  c->ppr = nullptr;
  cudaFree(c->wk);
  cudaFree(c->rho);
  for (int p = 0; p < 2; ++p) { cudaFree(c->e32[p]); cudaFree(c->ce32[p]); }
  cudaFree(c->batch);
  cudaFree(c->st);
  cudaFreeHost(c->st_host);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->tev) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  delete c;
  return PRX_OK;
}

void* prx_context_stream(prx_context* c) { return c ? (void*)c->stream : nullptr; }

}  // extern "C"

// ---- workspace -------------------------------------------------------------------
int ensure_ws(prx_context* c, uint32_t n, bool dyn) {
  if (c->ws_n >= n && (c->ws_dyn || !dyn)) return PRX_OK;
  const uint32_t cap = std::max(n, c->ws_n);
  const bool want_dyn = dyn || c->ws_dyn;
  free_ws(c);
  const size_t words = ((size_t)cap + 31) / 32;
  for (int p = 0; p < 2; ++p) {
    TRY_CUDA_ST(cudaMalloc(&c->r[p], sizeof(double) * cap));
    TRY_CUDA_ST(cudaMalloc(&c->c[p], sizeof(double) * cap));
  }
  TRY_CUDA_ST(cudaMalloc(&c->acc64, sizeof(double) * cap));
  TRY_CUDA_ST(cudaMalloc(&c->acc32, sizeof(float) * cap));
  if (want_dyn) {
    TRY_CUDA_ST(cudaMalloc(&c->flags, cap));
    for (auto& b : c->bm) TRY_CUDA_ST(cudaMalloc(&b, sizeof(uint32_t) * words));
    for (auto& b : c->nf) TRY_CUDA_ST(cudaMalloc(&b, sizeof(uint32_t) * words));
    TRY_CUDA_ST(cudaMalloc(&c->xb, sizeof(uint32_t) * cap));
    TRY_CUDA_ST(cudaMalloc(&c->naff, sizeof(uint32_t) * words));
    TRY_CUDA_ST(cudaMalloc(&c->ever, sizeof(uint32_t) * words));
    TRY_CUDA_ST(cudaMalloc(&c->pf, sizeof(double) * ((size_t)cap + kPfTable)));  // + the per-degree table
    TRY_CUDA_ST(cudaMalloc(&c->xl, sizeof(uint32_t) * cap));
    for (auto& f : c->fr) TRY_CUDA_ST(cudaMalloc(&f, sizeof(uint32_t) * cap));
    for (int k = MID; k < NCLS; ++k) TRY_CUDA_ST(cudaMalloc(&c->lists[0][k], sizeof(uint32_t) * cap));
  }
  c->ws_n = cap;
  c->ws_dyn = want_dyn;
  return PRX_OK;
}

int ensure_ch(prx_context* c, uint32_t hot_n) {
  if (c->ch_n >= hot_n) return PRX_OK;
  for (auto& h : c->ch) { cudaFree(h); h = nullptr; }
  c->ch_n = 0;
  for (auto& h : c->ch) TRY_CUDA_ST(cudaMalloc(&h, sizeof(double) * hot_n));
  c->ch_n = hot_n;
  return PRX_OK;
}

static int ensure_ws32(prx_context* c, uint32_t n) {
  if (c->ws32_n >= n) return PRX_OK;
  cudaFree(c->rho);
  c->rho = nullptr;
  for (int p = 0; p < 2; ++p) {
    cudaFree(c->e32[p]); c->e32[p] = nullptr;
    cudaFree(c->ce32[p]); c->ce32[p] = nullptr;
  }
  c->ws32_n = 0;
  TRY_CUDA_ST(cudaMalloc(&c->rho, sizeof(float) * n));
  for (int p = 0; p < 2; ++p) {
    TRY_CUDA_ST(cudaMalloc(&c->e32[p], sizeof(float) * n));
    TRY_CUDA_ST(cudaMalloc(&c->ce32[p], sizeof(float) * n));
  }
  c->ws32_n = n;
  return PRX_OK;
}

static int ensure_batch(prx_context* c, size_t elems) {
  if (c->batch_cap >= elems) return PRX_OK;
  cudaFree(c->batch);
  c->batch = nullptr;
  c->batch_cap = 0;
  TRY_CUDA_ST(cudaMalloc(&c->batch, sizeof(uint32_t) * std::max<size_t>(elems, 1024)));
  c->batch_cap = std::max<size_t>(elems, 1024);
  return PRX_OK;
}

SolveArgs make_args(prx_context* c, const GraphDev& g, const prx_options& o) {
  SolveArgs a;
  std::memset(&a, 0, sizeof(a));
  a.xoff = g.xoff; a.xedg = g.xedg;
  a.xtoff = g.xtoff; a.xtedg = g.xtedg; a.xtdat = g.xtdat;
  a.xbase = g.xbase; a.xtbase = g.xtbase; a.seg_shift = g.seg_shift;
  a.cls_list = g.cls_list;
  for (int k = 0; k < 3; ++k) a.fr[k] = c->fr[k];
  for (int p = 0; p < 2; ++p) {
    a.r[p] = c->r[p];
    a.c[p] = c->c[p];
    a.ch[p] = c->ch[p];
    for (int k = 0; k < NCLS; ++k) a.list[p][k] = c->lists[p][k];
  }
  for (int k = 0; k < 3; ++k) a.bm[k] = c->bm[k];
  a.nf[0] = c->nf[0]; a.nf[1] = c->nf[1];
  a.naff = c->naff; a.xl = c->xl; a.xb = c->xb;
  a.rho = c->rho;
  for (int p = 0; p < 2; ++p) { a.e[p] = c->e32[p]; a.ce[p] = c->ce32[p]; }
  a.low_bm = g.low_bm;
  a.rcp = g.rcp;
  a.ever = c->ever;
  a.pf = c->pf;
  a.pf_tab = c->pf ? c->pf + c->ws_n : nullptr;
  a.acc64 = c->acc64;
  a.acc32 = c->acc32;
  // expand by pulling once more than 1/16 of the vertices changed by > D
  a.pull_threshold = o.expansion == 1 ? 0xffffffffu : (o.expansion == 2 ? 0u : g.n / 16);
  // int_adds: the option, else the autotuner's pick, else the library default
  const int ia = o.int_adds ? o.int_adds : (g.tuned_int_adds ? g.tuned_int_adds : (int)kDefaultIntAdds);
  a.int_adds = ia > 0 ? (uint32_t)ia : 0u;
  a.st = c->st;
  a.n = g.n;
  a.mid_max = g.mid_max;
  a.P = o.damping;
  a.C0 = (1 - o.damping) / (double)g.n;  // pagerankLoopCuU :679, N = order
  a.D = o.frontier_tolerance;
  a.C = o.prune_tolerance;
  return a;
}

static bool valid_mode(int m) { return m >= PRX_STATIC && m <= PRX_PRUNE_DYNAMIC_FRONTIER; }

// Initial marking of a dynamic mode on batch arrays already on the device.
int run_marking(prx_context* c, const SolveArgs& a, int mode, const uint32_t* du, const uint32_t* dv,
                       uint64_t nd, const uint32_t* iu, uint64_t ni) {
  cudaStream_t s = c->stream;
  const size_t words = ((size_t)a.n + 31) / 32;
  for (auto b : c->bm) TRY_CUDA_ST(cudaMemsetAsync(b, 0, words * 4, s));
  for (auto b : c->nf) TRY_CUDA_ST(cudaMemsetAsync(b, 0, words * 4, s));
  TRY_CUDA_ST(cudaMemsetAsync(c->naff, 0, words * 4, s));
  if (nd + ni == 0) return PRX_OK;  // :927,956,985 -- nothing marked
  launch_mark_seed(a, du, dv, nd, iu, ni, c->sms, s);
  launch_expand_seeds(a, c->sms, s);
  launch_expand_big(a, 0, c->sms, s);
  c->launches += 3;
  TRY_CUDA_ST(cudaMemsetAsync(&c->st->xbcnt, 0, sizeof(uint32_t), s));
  if (mode == PRX_DYNAMIC_TRAVERSAL) {
    // The closure of the DF marking under out-edges.  A work queue of reached
    // vertices (k_closure_queue) runs it without levels, so a high-diameter
    // graph costs one launch instead of one per BFS level.  When the queue
    // explodes (more than pull_threshold vertices, n/16 by default, and eight
    // times those expanded), the closure is about to cover most of the graph:
    // the rest is done by pull rounds until one adds nothing -- each vertex
    // not yet reached scans its in-edges only until it finds a reached one,
    // so it no longer walks every out-edge.  prx_options.expansion 1 never
    // switches, 2 pulls from the start.  The set is the same either way.
    const size_t qbytes = sizeof(uint32_t) * (size_t)a.n;
    TRY_CUDA_ST(cudaMemsetAsync(c->fr[0], 0xff, qbytes, s));
    launch_frontier_from_bitmap(a, c->sms, s);
    c->launches += 1;
    bool pull = a.pull_threshold == 0;
    if (!pull) {
      launch_closure_queue(a, a.pull_threshold, c->sms, s);
      c->launches += 1;
      TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
      TRY_CUDA_ST(cudaStreamSynchronize(s));
      const State& h = c->st_host[1];
      if (h.err & kErrClosureWait) FAIL(PRX_ETIMEOUT, "DT closure: a bounded device wait ran out");
      pull = h.q_done != h.fcnt[0];  // left to pull rounds
    }
    if (pull) {
      // rounds in batches of 1, 2, 4, ..., 64; done when a round of the batch
      // returned early (pdone) or, all having run, the last one added nothing
      TRY_CUDA_ST(cudaMemsetAsync(c->st->pcnt, 0, sizeof(c->st->pcnt) + sizeof(c->st->pdone), s));
      uint32_t round = 0;
      for (uint32_t k = 1;; k = std::min<uint32_t>(2 * k, 64)) {
        for (uint32_t i = 0; i < k; ++i) launch_closure_pull(a, round++, c->sms, s);
        c->launches += k;
        TRY_CUDA_ST(cudaMemcpyAsync(c->st_host[1].pcnt, c->st->pcnt, sizeof(c->st->pcnt) + sizeof(c->st->pdone),
                                    cudaMemcpyDeviceToHost, s));
        TRY_CUDA_ST(cudaStreamSynchronize(s));
        if (c->st_host[1].pdone || c->st_host[1].pcnt[(round - 1) % 3] == 0) break;
      }
    }
  }
  TRY_CUDA_ST(cudaMemsetAsync(&c->st->xcnt, 0, sizeof(uint32_t), s));
  launch_popcount(c->bm[0], a.n, &c->st->affected, c->sms, s);
  c->launches += 1;
  return PRX_OK;
}

// Fold the recorded update-launch timings into the context's totals.
static int drain_timing(prx_context* c) {
  for (size_t i = 0; i < c->tev_used; ++i) {
    float ms = 0;
    TRY_CUDA_ST(cudaEventElapsedTime(&ms, c->tev[2 * i], c->tev[2 * i + 1]));
    c->upd_ms[c->tev_cls[i]] += ms;
    c->upd_n[c->tev_cls[i]] += 1;
  }
  c->tev_used = 0;
  return PRX_OK;
}

// Launch one rank-update kernel through `fn` (returns whether it launched),
// bracketed by CUDA events when timing; `slot` is its row in upd_ms.
template <class F>
static int launch_update_timed(prx_context* c, bool timing, int slot, F fn) {
  cudaStream_t s = c->stream;
  if (timing) {
    if (c->tev.size() < 2 * (c->tev_used + 1)) {
      cudaEvent_t e0, e1;
      TRY_CUDA_ST(cudaEventCreate(&e0));
      TRY_CUDA_ST(cudaEventCreate(&e1));
      c->tev.push_back(e0);
      c->tev.push_back(e1);
      c->tev_cls.push_back(0);
    }
    TRY_CUDA_ST(cudaEventRecord(c->tev[2 * c->tev_used], s));
  }
  const bool launched = fn();
  c->launches += launched;
  if (timing && launched) {
    TRY_CUDA_ST(cudaEventRecord(c->tev[2 * c->tev_used + 1], s));
    c->tev_cls[c->tev_used++] = slot;
  }
  return PRX_OK;
}

int enqueue_iteration(prx_context* c, const GraphDev& g, const SolveArgs& a, int mode, bool timing,
                      const ChunkLayout* lay) {
  cudaStream_t s = c->stream;
  for (int cls = 0; cls < NCLS; ++cls) {
    const int slot = (mode & MODE_F32) ? NCLS + cls : cls;  // FP32 sweeps are timed apart
    const int st = launch_update_timed(c, timing, slot,
                                       [&] { return launch_update_class(a, g, mode, cls, lay, c->sms, s); });
    if (st) return st;
  }
  // the contributions this iteration wrote (the dynamic modes' stale copies
  // included: after an iteration its parity holds every vertex's value)
  if (!(mode & MODE_F32)) c->launches += launch_hot_copy(a, -1, c->sms, s);
  if ((mode & ~MODE_F32) >= PRX_DYNAMIC_FRONTIER) {
    launch_expand_iteration(a, c->sms, s);  // push or pull, chosen on the device
    c->launches += 3;
  }
  launch_finalize(a, mode, s);
  c->launches += 1;
  return PRX_OK;
}

// ---- the iteration loop as one CUDA graph ----------------------------------
// A conditional WHILE node whose body is one iteration (the update launches,
// the expansion and k_finalize) followed by k_loop_cond, which keeps the loop
// going while the solve is not done.  k_loop_cond counts the bodies itself
// and stops after `cap` of them whatever the other kernels did, so the loop
// ends even if k_finalize never ran: at most max_iterations + 1 bodies run.
__global__ void k_loop_cond(cudaGraphConditionalHandle h, State* st, int cap) {
  const int rounds = ++st->graph_rounds;
  cudaGraphSetConditional(h, (!st->done && rounds < cap) ? 1u : 0u);
}

static int run_graph_loop(prx_context* c, const prx_graph* gr, const SolveArgs& a, int mode, const ChunkLayout* lay,
                          int max_iter) {
  cudaStream_t s = c->stream;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int st = PRX_OK;
  auto fail = [&](cudaError_t e, const char* what) {
    set_error(std::string("prx_solve (graph loop): ") + what + ": " + cudaGetErrorString(e));
    st = e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
  };
  cudaError_t e = cudaGraphCreate(&graph, 0);
  cudaGraphConditionalHandle h{};
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &p);
  const uint64_t l0 = c->launches;
  uint64_t per_body = 0;
  if (e == cudaSuccess) {
    cudaGraph_t body = p.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const int st_enq = enqueue_iteration(c, gr->g, a, mode, false, lay);
      const int cap = (max_iter < (1 << 30) ? max_iter : (1 << 30)) + 2;
      k_loop_cond<<<1, 1, 0, s>>>(h, a.st, cap);
      per_body = c->launches - l0 + 1;
      const cudaError_t e_launch = cudaGetLastError();
      cudaGraph_t captured = nullptr;
      e = cudaStreamEndCapture(s, &captured);  // always leave capture mode
      if (st_enq) st = st_enq;
      if (e == cudaSuccess) e = e_launch;
    }
  }
  if (e == cudaSuccess && !st) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess && !st) e = cudaGraphLaunch(exec, s);
  if (e == cudaSuccess && !st) e = cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && !st) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess && !st) fail(e, "build or launch");
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  c->launches = l0 + per_body * (uint64_t)(st ? 0 : c->st_host[1].graph_rounds);
  return st;
}

// FP32 refinement loop (prx_refine.cu).  *final_parity: 1 when the last FP64
// sweep converged (its output in r[1]), 0 when the cap stopped an FP32 round
// (the committed ranks in r[0]).
// The same loop as one CUDA graph launch: [round 0: k_refine_round0, an FP32
// round, commit] then WHILE (not done, under the cap) { FP64 residual sweep,
// k_refine_finalize64, WHILE (round not ended) { FP32 sweep, k_finalize32 },
// commit (nothing once done) }.  The answer: the last FP64 sweep's output when
// one of them ended the solve, else the committed ranks.
static int run_refine_graph(prx_context* c, const prx_graph* gr, const SolveArgs& a, int max_iter,
                            const ChunkLayout* lay64, const ChunkLayout* lay32, int* final_parity, bool round0) {
  cudaStream_t s = c->stream, s2 = nullptr, s3 = nullptr;
  const GraphDev& g = gr->g;
  const int cap = (max_iter < (1 << 30) ? max_iter : (1 << 30)) + 2;
  uint64_t l32 = 0, l64 = 0, lfix = 0;  // launches per FP32 body, per FP64 body, outside the loops
  auto fp32_body = [&](cudaStream_t sw, cudaGraphConditionalHandle h) -> cudaError_t {
    const uint64_t l0 = c->launches;
    for (int cls = 0; cls < NCLS; ++cls) c->launches += launch_sweep32(a, g, cls, lay32, c->sms, sw);
    launch_finalize32(a, sw);
    launch_refine_cond(h, a, true, cap, sw);
    l32 = c->launches - l0 + 2;
    return cudaGetLastError();
  };
  auto round_end = [&](cudaStream_t sw) {
    launch_refine_commit(a, c->sms, sw);
    launch_hot_copy(a, 0, c->sms, sw);
  };
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s3, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t ec = cudaSuccess;
    if (round0) {
      launch_refine_round0(a, c->sms, s);
      ec = capture_conditional(s, s2, cudaGraphCondTypeWhile, 0,
                               [&](cudaGraphConditionalHandle h) { launch_refine_arm(h, a, true, s); }, fp32_body);
      if (ec == cudaSuccess) round_end(s);
    }
    if (ec == cudaSuccess)
      ec = capture_conditional(
          s, s2, cudaGraphCondTypeWhile, 0, [&](cudaGraphConditionalHandle h) { launch_refine_arm(h, a, false, s); },
          [&](cudaStream_t sb, cudaGraphConditionalHandle ho) -> cudaError_t {
            const uint64_t l0 = c->launches;
            for (int cls = 0; cls < NCLS; ++cls) c->launches += launch_refine_sweep64(a, g, cls, lay64, c->sms, sb);
            launch_refine_finalize64(a, sb);
            l64 = c->launches - l0 + 1;
            cudaError_t eb = capture_conditional(
                sb, s3, cudaGraphCondTypeWhile, 0,
                [&](cudaGraphConditionalHandle h) { launch_refine_arm(h, a, true, sb); }, fp32_body);
            if (eb != cudaSuccess) return eb;
            round_end(sb);
            launch_refine_cond(ho, a, false, cap, sb);
            return cudaGetLastError();
          });
    const cudaError_t el = cudaGetLastError();
    e = cudaStreamEndCapture(s, &graph);  // always leave capture mode
    if (e == cudaSuccess) e = ec;
    if (e == cudaSuccess) e = el;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (s2) cudaStreamDestroy(s2);
  if (s3) cudaStreamDestroy(s3);
  TRY_CUDA_ST(e);
  const State& h = c->st_host[1];
  lfix = round0 ? 3 : 0;  // round 0, commit, hot copy
  c->launches += lfix + (uint64_t)h.rounds * (l64 + 2) + (uint64_t)(h.iter - h.rounds) * l32;
  // the FP64 sweep's output is the answer only when one of the outer loop's
  // sweeps ended the solve (done may also be set on entry, by the cap)
  *final_parity = (h.graph_rounds > 0 && h.done) ? 1 : 0;
  return PRX_OK;
}

static int run_refine_loop(prx_context* c, const prx_graph* gr, const SolveArgs& a, bool timing, int max_iter,
                           const ChunkLayout* lay64, const ChunkLayout* lay32, int* final_parity, bool round0,
                           bool graph) {
  cudaStream_t s = c->stream;
  int st;
  if (graph && !timing && max_iter > 0) return run_refine_graph(c, gr, a, max_iter, lay64, lay32, final_parity, round0);
  // one round of FP32 correction sweeps until they stop, then x_b += e
  auto fp32_round = [&]() -> int {
    for (int k = 1;; k = std::min(2 * k, 16)) {
      for (int i = 0; i < k; ++i) {
        for (int cls = 0; cls < NCLS; ++cls) {
          st = launch_update_timed(c, timing, NCLS + cls,
                                   [&] { return launch_sweep32(a, gr->g, cls, lay32, c->sms, s); });
          if (st) return st;
        }
        launch_finalize32(a, s);
        c->launches += 1;
      }
      TRY_CUDA_ST(cudaGetLastError());
      TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
      TRY_CUDA_ST(cudaStreamSynchronize(s));
      if (timing && (st = drain_timing(c))) return st;
      if (c->st_host[1].inner_done) break;
    }
    launch_refine_commit(a, c->sms, s);
    c->launches += 1 + launch_hot_copy(a, 0, c->sms, s);
    return PRX_OK;
  };
  if (max_iter <= 0) {
    TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
    TRY_CUDA_ST(cudaStreamSynchronize(s));
    *final_parity = 0;  // no sweep: the initial ranks
    return PRX_OK;
  }
  // round 0: FP32 sweeps of the ranks themselves from the initial ranks (the
  // dynamic modes start from the committed result of their FP32 phase instead)
  if (round0) {
    launch_refine_round0(a, c->sms, s);
    c->launches += 1;
    if ((st = fp32_round())) return st;
  } else {
    TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
    TRY_CUDA_ST(cudaStreamSynchronize(s));
  }
  if (c->st_host[1].iter >= max_iter) {
    TRY_CUDA_ST(cudaStreamSynchronize(s));
    *final_parity = 0;
    return PRX_OK;
  }
  for (;;) {
    for (int cls = 0; cls < NCLS; ++cls) {
      st = launch_update_timed(c, timing, cls,
                               [&] { return launch_refine_sweep64(a, gr->g, cls, lay64, c->sms, s); });
      if (st) return st;
    }
    launch_refine_finalize64(a, s);
    c->launches += 1;
    TRY_CUDA_ST(cudaGetLastError());
    TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
    TRY_CUDA_ST(cudaStreamSynchronize(s));
    if (timing && (st = drain_timing(c))) return st;
    if (c->st_host[1].done) {  // converged (or capped) at this FP64 sweep: its output
      *final_parity = 1;
      return PRX_OK;
    }
    if ((st = fp32_round())) return st;
    if (c->st_host[1].iter >= max_iter) {
      TRY_CUDA_ST(cudaStreamSynchronize(s));
      *final_parity = 0;
      return PRX_OK;
    }
  }
}

// Core solve; q_dev/batch arrays are device pointers.  On success *final_ranks
// points at the device buffer holding the ranks.
static int solve_core(prx_context* c, prx_graph* gr, int mode, const uint32_t* du, const uint32_t* dv, uint64_t nd,
                      const uint32_t* iu, uint64_t ni, const double* q_dev, const prx_options& o,
                      prx_result* res, const double** final_ranks) {
  const GraphDev& g = gr->g;
  const bool dyn = mode >= PRX_DYNAMIC_TRAVERSAL;
  if (dyn && !g.xoff) FAIL(PRX_ESTATE, "prx_solve: dynamic modes need the out-CSR (xoff/xedg) of the graph");
  if (o.precision != PRX_FP64 && o.precision != PRX_FP32_REFINE) FAIL(PRX_EINVAL, "prx_solve: unknown precision");
  const bool refine = o.precision == PRX_FP32_REFINE;
  int st = ensure_ws(c, g.n, dyn);
  if (st) return st;
  if (refine && (st = ensure_ws32(c, g.n))) return st;
  int final_parity = -1;
  // source-chunk layouts of the LOW gathers, built once per graph version and
  // width.  Defaults from a width sweep on the 50M-vertex web-like graph: the
  // FP64 sweep (bound by GB300's FP64 add rate as much as by HBM) gains from
  // two chunks only (200 MB of contributions each), the FP32 sweep from
  // 48 MB chunks.
  const uint32_t w64 = o.chunk_vertices ? o.chunk_vertices
                      : g.tuned_w64          ? g.tuned_w64
                                             : kDefaultChunk64;
  const uint32_t w32 = o.chunk_vertices ? o.chunk_vertices
                      : g.tuned_w32          ? g.tuned_w32
                                             : (48u << 20) / sizeof(float);
  // Hot sources (the FP64 sweeps of every mode): a layout whose edges from
  // the highest out-degree vertices gather from a dense copy of their
  // contributions
  const bool hot_ok = o.hot_sources >= 0;
  if (hot_ok) {
    TRY_CUDA_ST(ensure_hot(gr->g, o.hot_sources > 0 ? (uint32_t)o.hot_sources : kDefaultHotCap, c->sms,
                           c->stream));
    if (g.hot_n && (st = ensure_ch(c, g.hot_n))) return st;
  }
  const ChunkLayout *lay64 = nullptr, *lay32 = nullptr;
  TRY_CUDA_ST(ensure_chunks(gr->g, w64, c->sms, c->stream, &lay64, hot_ok && g.hot_n > 0));
  if (refine) TRY_CUDA_ST(ensure_chunks(gr->g, w32, c->sms, c->stream, &lay32));
  cudaStream_t s = c->stream;
  SolveArgs a = make_args(c, g, o);
  a.hot_list = g.hot_list;
  a.hot_n = (lay64 && lay64->hot) ? g.hot_n : 0;
  const int repeat = o.repeat > 0 ? o.repeat : 1;
  float ti = 0, tm = 0, tc = 0, tt = 0;
  const bool timing = o.timing != 0;
  bool full_sweeps = false;  // FP32-refined dynamic mode run as full sweeps (last repeat)
  bool dt_all = false;       // DT whose closure covers every vertex, run as ND (last repeat)
  for (int rep = 0; rep < repeat; ++rep) {
    c->launches = 0;
    c->tev_used = 0;
    for (int k = 0; k < 2 * NCLS; ++k) { c->upd_ms[k] = 0; c->upd_n[k] = 0; }
    TRY_CUDA_ST(cudaEventRecord(c->ev[0], s));
    launch_state_reset(c->st, o.max_iterations, o.tolerance, s);
    launch_init_ranks(a, (mode == PRX_STATIC) ? nullptr : q_dev, dyn, s);
    c->launches += 2 + launch_hot_copy(a, 0, c->sms, s);
    if (mode == PRX_PRUNE_DYNAMIC_FRONTIER && !refine) {
      launch_prune_factor(a, s);
      c->launches += 1;
    }
    if (refine && dyn) {
      launch_init_ranks32(a, q_dev, s);
      TRY_CUDA_ST(cudaMemsetAsync(c->ever, 0, sizeof(uint32_t) * (((size_t)g.n + 31) / 32), s));
      c->launches += 1;
    }
    TRY_CUDA_ST(cudaEventRecord(c->ev[1], s));
    if (dyn) {
      st = run_marking(c, a, mode, du, dv, nd, iu, ni);
      if (st) return st;
      TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[0], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
    }
    TRY_CUDA_ST(cudaEventRecord(c->ev[2], s));
    // iterations of `m` until done: one CUDA graph, or host-driven batches
    auto iterate = [&](int m, const ChunkLayout* lay) -> int {
      if (o.loop != PRX_LOOP_HOST && !timing) return run_graph_loop(c, gr, a, m, lay, o.max_iterations);
      for (int k = 1;; k = std::min(2 * k, 16)) {
        for (int i = 0; i < k; ++i) {
          const int e = enqueue_iteration(c, gr->g, a, m, timing, lay);
          if (e) return e;
        }
        TRY_CUDA_ST(cudaGetLastError());
        TRY_CUDA_ST(cudaMemcpyAsync(&c->st_host[1], c->st, sizeof(State), cudaMemcpyDeviceToHost, s));
        TRY_CUDA_ST(cudaStreamSynchronize(s));
        if (timing) {
          const int e = drain_timing(c);
          if (e) return e;
        }
        if (c->st_host[1].done) return PRX_OK;
      }
    };
    // DT whose closure reached every vertex updates every vertex in every
    // iteration with nothing to expand or prune: exactly ND's iterations,
    // which the Static kernels run without the bitmaps
    dt_all = false;
    if (mode == PRX_DYNAMIC_TRAVERSAL && !refine && nd + ni > 0) {
      TRY_CUDA_ST(cudaStreamSynchronize(s));
      dt_all = c->st_host[0].affected == g.n;
    }
    full_sweeps = refine && dyn && o.refine_sweeps == 1;
    if (refine && dyn && o.refine_sweeps == 0) {  // the initial marking's size decides
      TRY_CUDA_ST(cudaStreamSynchronize(s));
      full_sweeps = c->st_host[0].affected > g.n / 8;
    }
    if (refine && dyn && !full_sweeps) {
      // DT / DF / DF-P with FP32 ranks, then the FP64 refinement of the result
      // (an FP64 residual sweep over all vertices decides convergence)
      if ((st = iterate(mode | MODE_F32, lay32))) return st;
      launch_commit_dyn32(a, c->st_host[1].iter & 1, s);
      c->launches += 1 + launch_hot_copy(a, 0, c->sms, s);
      if ((st = run_refine_loop(c, gr, a, timing, o.max_iterations, lay64, lay32, &final_parity, false,
                                o.loop != PRX_LOOP_HOST)))
        return st;
    } else if (refine) {
      // Static / ND, or a dynamic mode whose marking covers most of the
      // graph: FP32 sweeps over all vertices from the initial ranks (q for
      // the dynamic modes), then the FP64 refinement
      if ((st = run_refine_loop(c, gr, a, timing, o.max_iterations, lay64, lay32, &final_parity, true,
                                o.loop != PRX_LOOP_HOST)))
        return st;
    } else if ((st = iterate(dt_all ? PRX_NAIVE_DYNAMIC : mode, lay64))) {
      return st;
    }
    TRY_CUDA_ST(cudaEventRecord(c->ev[3], s));
    TRY_CUDA_ST(cudaEventSynchronize(c->ev[3]));
    float x;
    cudaEventElapsedTime(&x, c->ev[0], c->ev[1]); ti += x;
    cudaEventElapsedTime(&x, c->ev[1], c->ev[2]); tm += x;
    cudaEventElapsedTime(&x, c->ev[2], c->ev[3]); tc += x;
    cudaEventElapsedTime(&x, c->ev[0], c->ev[3]); tt += x;
  }
  const State& h = c->st_host[1];
  if (res) {
    res->iterations = h.iter;
    res->time_ms = tt / repeat;
    res->initialization_time_ms = ti / repeat;
    res->marking_time_ms = tm / repeat;
    res->computation_time_ms = tc / repeat;
    res->affected_initial = dyn ? c->st_host[0].affected : g.n;
    res->edges_processed = dyn && !full_sweeps && !dt_all ? h.edges : g.m * (uint64_t)h.iter;
    res->last_delta = h.last_delta;
    res->refinements = refine ? h.rounds : 0;
    res->kernel_launches = c->launches;
    for (int k = 0; k < NCLS; ++k) {
      res->update_ms[k] = c->upd_ms[k];
      res->update_launches[k] = c->upd_n[k];
      res->update32_ms[k] = c->upd_ms[NCLS + k];
      res->update32_launches[k] = c->upd_n[NCLS + k];
    }
  }
  *final_ranks = refine ? c->r[final_parity] : c->r[h.iter & 1];
  return PRX_OK;
}

// Segmented 32-bit offsets from 64-bit ones: entry i of segment k (rows
// [k * 2^S, ...), 2^S + 1 entries each) is off64[v] - off64[k * 2^S] with
// v = k * 2^S + i.
__global__ void k_segment_offsets(const unsigned long long* __restrict__ off64, uint32_t n, uint32_t shift,
                                  uint64_t entries, uint32_t* __restrict__ off) {
  const uint64_t per = (1ull << shift) + 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < entries; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = i / per, j = i - k * per;
    const uint64_t v = (k << shift) + j;
    off[i] = v <= n ? (uint32_t)(off64[v] - off64[k << shift]) : 0u;
  }
}

// Row segments for 64-bit offsets (see GraphDev): the largest shift <= 30
// whose segments all hold fewer than 2^32 - 8 edges in every CSR given, or
// `want` if it is not 0; 32 (one segment) when m < 2^32 and want is 0.
static int pick_shift(uint32_t n, uint64_t m, const uint64_t* a, const uint64_t* b, uint32_t want, uint32_t* out) {
  auto fits = [&](uint32_t S) {
    if (S >= 32) return m < 0xfffffff8ull;
    for (uint64_t v0 = 0; v0 < n; v0 += 1ull << S) {
      const uint64_t v1 = std::min<uint64_t>(n, v0 + (1ull << S));
      if (a[v1] - a[v0] >= 0xfffffff8ull) return false;
      if (b && b[v1] - b[v0] >= 0xfffffff8ull) return false;
    }
    return true;
  };
  if (want) {
    if (want > 32 || !fits(want)) FAIL(PRX_ERANGE, "prx_graph_create64: a row segment holds 2^32 edges or more");
    *out = want;
    return PRX_OK;
  }
  if (fits(32)) {
    *out = 32;
    return PRX_OK;
  }
  for (uint32_t S = 30; S >= 1; --S)
    if (fits(S)) {
      *out = S;
      return PRX_OK;
    }
  FAIL(PRX_ERANGE, "prx_graph_create64: a row holds 2^32 edges or more");
}

static int check_batch_ids(uint32_t n, const uint32_t* du, const uint32_t* dv, uint64_t nd, const uint32_t* iu,
                           const uint32_t* iv, uint64_t ni) {
  if ((nd && (!du || !dv)) || (ni && !iu)) FAIL(PRX_EINVAL, "batch: NULL array with a non-zero length");
  for (uint64_t i = 0; i < nd; ++i)
    if (du[i] >= n || dv[i] >= n) FAIL(PRX_EINVAL, "batch: deletion vertex id out of range");
  for (uint64_t i = 0; i < ni; ++i)
    if (iu[i] >= n || (iv && iv[i] >= n)) FAIL(PRX_EINVAL, "batch: insertion vertex id out of range");
  return PRX_OK;
}

extern "C" {

int prx_graph_create(prx_context* c, uint32_t n, uint64_t m, const uint32_t* xoff, const uint32_t* xedg,
                     const uint32_t* xtoff, const uint32_t* xtedg, const uint32_t* xtdat, int validate,
                     prx_graph** out) {
  if (!c || !out) FAIL(PRX_EINVAL, "prx_graph_create: NULL context or out");
  *out = nullptr;
  if (m > 0xffffffffull) FAIL(PRX_ERANGE, "prx_graph_create: m >= 2^32 does not fit 32-bit offsets");
  if (n > kMaxVertices) FAIL(PRX_ERANGE, "prx_graph_create: more than 2^32 - 2^24 vertices");
  if (!xtoff || (n && !xtdat) || (m && !xtedg))
    FAIL(PRX_EINVAL, "prx_graph_create: xtoff, xtedg and xtdat are required");
  if ((xedg && !xoff) || (xoff && m && !xedg)) FAIL(PRX_EINVAL, "prx_graph_create: give both xoff and xedg or neither");
  if (xtoff[0] != 0 || xtoff[n] != m) FAIL(PRX_EINVAL, "prx_graph_create: xtoff must start at 0 and end at m");
  if (xoff && (xoff[0] != 0 || xoff[n] != m)) FAIL(PRX_EINVAL, "prx_graph_create: xoff must start at 0 and end at m");
  if (validate) {
    for (uint32_t v = 0; v < n; ++v) {
      if (xtoff[v + 1] < xtoff[v]) FAIL(PRX_EINVAL, "prx_graph_create: xtoff not monotone");
      if (xoff && xoff[v + 1] < xoff[v]) FAIL(PRX_EINVAL, "prx_graph_create: xoff not monotone");
      if (xoff && xtdat[v] != xoff[v + 1] - xoff[v]) FAIL(PRX_EINVAL, "prx_graph_create: xtdat != out-degree");
    }
    for (uint64_t i = 0; i < m; ++i) {
      if (xtedg[i] >= n) FAIL(PRX_EINVAL, "prx_graph_create: xtedg id out of range");
      if (xedg && xedg[i] >= n) FAIL(PRX_EINVAL, "prx_graph_create: xedg id out of range");
    }
  }
  TRY_CUDA_ST(cudaSetDevice(c->device));
  prx_graph* gr = new prx_graph();
  gr->ctx = c;
  GraphDev& g = gr->g;
  g.device = c->device;
  g.n = n;
  g.m = m;
  g.m_cap = m;
  cudaStream_t s = c->stream;
  // The in-edges go up on a copy stream in row-range pieces; meanwhile the
  // degree classes, the hot sources and the default LOW layout are built on
  // the context's stream, each piece's part of the layout as soon as that
  // piece has landed.  The out-CSR (dynamic modes) follows the in-edges.
  auto alloc = [&](uint32_t** dst, size_t cnt, size_t slots = 0) -> cudaError_t {
    return graph_alloc(dst, sizeof(uint32_t) * (slots > cnt ? slots : (cnt ? cnt : 1)), s);
  };
  cudaError_t e = alloc(&g.xtoff, (size_t)n + 1);
  if (e == cudaSuccess) e = alloc(&g.xtedg, m, edge_slots(m));
  if (e == cudaSuccess) e = alloc(&g.xtdat, n);
  if (e == cudaSuccess && xoff) e = alloc(&g.xoff, (size_t)n + 1);
  if (e == cudaSuccess && xoff) e = alloc(&g.xedg, m);
  if (e == cudaSuccess && !c->copy_stream) e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
  constexpr int kMaxPieces = 8;
  const int pieces = (int)std::max<uint64_t>(1, std::min<uint64_t>(kMaxPieces, m >> 24));
  uint32_t rows[kMaxPieces + 1];
  rows[0] = 0;
  for (int p = 1; p < pieces; ++p) {  // piece p starts at the first row whose edges reach p/pieces of m (32-row steps)
    const uint64_t want = m * (uint64_t)p / pieces;
    uint32_t lo = rows[p - 1], hi = n;
    while (lo < hi) {
      const uint32_t mid = lo + (hi - lo) / 2;
      if (xtoff[mid] < want) lo = mid + 1; else hi = mid;
    }
    rows[p] = std::max(rows[p - 1], lo & ~31u);
  }
  rows[pieces] = n;
  cudaEvent_t ev[kMaxPieces + 3] = {};
  for (int i = 0; i < pieces + 3 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
  cudaEvent_t ev_alloc = ev[pieces], ev_meta = ev[pieces + 1], ev_done = ev[pieces + 2];
  cudaStream_t cs = c->copy_stream;
  auto h2d = [&](uint32_t* dst, const uint32_t* src, size_t cnt) -> cudaError_t {
    return cnt ? cudaMemcpyAsync(dst, src, sizeof(uint32_t) * cnt, cudaMemcpyHostToDevice, cs) : cudaSuccess;
  };
  if (e == cudaSuccess) e = cudaEventRecord(ev_alloc, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev_alloc, 0);
  if (e == cudaSuccess) e = h2d(g.xtoff, xtoff, (size_t)n + 1);
  if (e == cudaSuccess) e = h2d(g.xtdat, xtdat, n);
  if (e == cudaSuccess) e = cudaEventRecord(ev_meta, cs);
  for (int p = 0; p < pieces && e == cudaSuccess; ++p) {
    const uint32_t b = xtoff[rows[p]], en = xtoff[rows[p + 1]];
    e = h2d(g.xtedg + b, xtedg + b, en - b);
    if (e == cudaSuccess) e = cudaEventRecord(ev[p], cs);
  }
  if (e == cudaSuccess && xoff) e = h2d(g.xoff, xoff, (size_t)n + 1);
  if (e == cudaSuccess && xoff) e = h2d(g.xedg, xedg, m);
  if (e == cudaSuccess) e = cudaEventRecord(ev_done, cs);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev_meta, 0);
  if (e == cudaSuccess) e = build_classes(g, c->sms, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = tune_apply_cached(g, c->sms, s);
  if (e == cudaSuccess) e = ensure_hot(g, kDefaultHotCap, c->sms, s);
  if (e == cudaSuccess) {
    const uint32_t width = g.tuned_w64 ? g.tuned_w64 : kDefaultChunk64;
    e = build_default_layout_pipelined(g, width, g.hot_n > 0, pieces, rows, ev, c->sms, s);
  }
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev_done, 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) cudaStreamSynchronize(cs);  // no copy may still write into freed arrays
  for (auto x : ev)
    if (x) cudaEventDestroy(x);
  if (e != cudaSuccess) {
    set_error(std::string("prx_graph_create: ") + cudaGetErrorString(e));
    prx_graph_destroy(gr);
    return e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
  }
  *out = gr;
  return PRX_OK;
}

int prx_release_cached_memory(int device) {
  TRY_CUDA_ST(cudaSetDevice(device));
  TRY_CUDA_ST(cudaDeviceSynchronize());
  TRY_CUDA_ST(graph_pool_trim(device));
  return PRX_OK;
}

int prx_graph_pool_stats(int device, uint64_t* reserved, uint64_t* reserved_peak, uint64_t* used,
                         uint64_t* used_peak) {
  TRY_CUDA_ST(cudaSetDevice(device));
  uint64_t v[4];
  TRY_CUDA_ST(graph_pool_stats(device, v));
  if (reserved) *reserved = v[0];
  if (reserved_peak) *reserved_peak = v[1];
  if (used) *used = v[2];
  if (used_peak) *used_peak = v[3];
  return PRX_OK;
}

int prx_l2_fetch_granularity(int device, int bytes, int* previous) {
  if (bytes > 128) FAIL(PRX_EINVAL, "prx_l2_fetch_granularity: at most 128 bytes");
  TRY_CUDA_ST(cudaSetDevice(device));
  size_t cur = 0;
  TRY_CUDA_ST(cudaDeviceGetLimit(&cur, cudaLimitMaxL2FetchGranularity));
  if (previous) *previous = (int)cur;
  if (bytes >= 0) TRY_CUDA_ST(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)bytes));
  return PRX_OK;
}

int prx_graph_create64(prx_context* c, uint32_t n, uint64_t m, const uint64_t* xoff, const uint32_t* xedg,
                       const uint64_t* xtoff, const uint32_t* xtedg, const uint32_t* xtdat, int validate,
                       uint32_t seg_shift, prx_graph** out) {
  if (!c || !out) FAIL(PRX_EINVAL, "prx_graph_create64: NULL context or out");
  *out = nullptr;
  if (n > kMaxVertices) FAIL(PRX_ERANGE, "prx_graph_create64: more than 2^32 - 2^24 vertices");
  if (!xtoff || (n && !xtdat) || (m && !xtedg))
    FAIL(PRX_EINVAL, "prx_graph_create64: xtoff, xtedg and xtdat are required");
  if ((xedg && !xoff) || (xoff && m && !xedg)) FAIL(PRX_EINVAL, "prx_graph_create64: give both xoff and xedg or neither");
  if (xtoff[0] != 0 || xtoff[n] != m) FAIL(PRX_EINVAL, "prx_graph_create64: xtoff must start at 0 and end at m");
  if (xoff && (xoff[0] != 0 || xoff[n] != m)) FAIL(PRX_EINVAL, "prx_graph_create64: xoff must start at 0 and end at m");
  if (validate) {
    for (uint32_t v = 0; v < n; ++v) {
      if (xtoff[v + 1] < xtoff[v]) FAIL(PRX_EINVAL, "prx_graph_create64: xtoff not monotone");
      if (xoff && xoff[v + 1] < xoff[v]) FAIL(PRX_EINVAL, "prx_graph_create64: xoff not monotone");
      if (xoff && xtdat[v] != xoff[v + 1] - xoff[v]) FAIL(PRX_EINVAL, "prx_graph_create64: xtdat != out-degree");
    }
    for (uint64_t i = 0; i < m; ++i) {
      if (xtedg[i] >= n) FAIL(PRX_EINVAL, "prx_graph_create64: xtedg id out of range");
      if (xedg && xedg[i] >= n) FAIL(PRX_EINVAL, "prx_graph_create64: xedg id out of range");
    }
  }
  uint32_t S = 32;
  int st = pick_shift(n, m, xtoff, xoff, seg_shift, &S);
  if (st) return st;
  TRY_CUDA_ST(cudaSetDevice(c->device));
  prx_graph* gr = new prx_graph();
  gr->ctx = c;
  GraphDev& g = gr->g;
  g.device = c->device;
  g.n = n;
  g.m = g.m_cap = m;
  g.seg_shift = S;
  g.nseg = n ? (uint32_t)(((uint64_t)n + (1ull << S) - 1) >> S) : 1;
  if (S >= 32) g.nseg = 1;
  cudaStream_t s = c->stream;
  const uint64_t entries = (uint64_t)n + g.nseg;
  unsigned long long* tmp = nullptr;
  // one CSR: segment bases (edge positions rounded up to 16 bytes), offsets, edges
  auto build = [&](const uint64_t* off64, const uint32_t* edg, uint32_t** doff, uint32_t** dedg,
                   unsigned long long** dbase, std::vector<uint64_t>& seg0, std::vector<uint64_t>& pos) -> cudaError_t {
    seg0.assign(g.nseg, 0);
    pos.assign(g.nseg, 0);
    uint64_t slots = 0;
    for (uint32_t k = 0; k < g.nseg; ++k) {
      const uint64_t v0 = std::min<uint64_t>(n, (uint64_t)k << (S >= 32 ? 0 : S));
      seg0[k] = off64[S >= 32 ? 0 : v0];
      pos[k] = (slots + 3) & ~3ull;
      const uint64_t v1 = S >= 32 ? n : std::min<uint64_t>(n, v0 + (1ull << S));
      slots = pos[k] + (off64[v1] - seg0[k]);
    }
    cudaError_t e = graph_alloc(doff, 4 * entries, s);
    if (e == cudaSuccess) e = graph_alloc(dedg, 4 * (((slots + 3) & ~3ull) + 4), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tmp, off64, 8 * ((uint64_t)n + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      k_segment_offsets<<<c->sms * 8, 256, 0, s>>>(tmp, n, S >= 32 ? 63 : S, entries, *doff);
    for (uint32_t k = 0; k < g.nseg && e == cudaSuccess; ++k) {
      const uint64_t v0 = S >= 32 ? 0 : std::min<uint64_t>(n, (uint64_t)k << S);
      const uint64_t v1 = S >= 32 ? n : std::min<uint64_t>(n, v0 + (1ull << S));
      const uint64_t cnt = off64[v1] - off64[v0];
      if (cnt) e = cudaMemcpyAsync(*dedg + pos[k], edg + off64[v0], 4 * cnt, cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess && g.nseg > 1) {
      e = graph_alloc(dbase, 8 * (uint64_t)g.nseg, s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(*dbase, pos.data(), 8 * (uint64_t)g.nseg, cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host arrays above are the caller's
    return e;
  };
  cudaError_t e = cudaMalloc(&tmp, 8 * ((uint64_t)n + 1));
  if (e == cudaSuccess) e = build(xtoff, xtedg, &g.xtoff, &g.xtedg, &g.xtbase, g.xtseg0, g.xtpos);
  if (e == cudaSuccess && xoff) e = build(xoff, xedg, &g.xoff, &g.xedg, &g.xbase, g.xseg0, g.xpos);
  if (e == cudaSuccess) e = graph_alloc(&g.xtdat, 4 * (uint64_t)(n ? n : 1), s);
  if (e == cudaSuccess && n) e = cudaMemcpyAsync(g.xtdat, xtdat, 4 * (uint64_t)n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = build_classes(g, c->sms, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = tune_apply_cached(g, c->sms, s);
  cudaFree(tmp);
  if (e != cudaSuccess) {
    set_error(std::string("prx_graph_create64: ") + cudaGetErrorString(e));
    prx_graph_destroy(gr);
    return e == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;
  }
  *out = gr;
  return PRX_OK;
}

int prx_graph_download64(prx_graph* gr, uint64_t* xoff, uint32_t* xedg, uint64_t* xtoff, uint32_t* xtedg,
                         uint32_t* xtdat) {
  if (!gr) FAIL(PRX_EINVAL, "prx_graph_download64: NULL graph");
  const GraphDev& g = gr->g;
  cudaStream_t s = gr->ctx->stream;
  TRY_CUDA_ST(cudaSetDevice(gr->ctx->device));
  if ((xoff || xedg) && !g.xoff) FAIL(PRX_ESTATE, "prx_graph_download64: graph has no out-CSR");
  const uint64_t entries = (uint64_t)g.n + g.nseg;
  std::vector<uint32_t> rel(entries);
  auto one = [&](const uint32_t* doff, const uint32_t* dedg, const std::vector<uint64_t>& seg0,
                 const std::vector<uint64_t>& pos, uint64_t* off, uint32_t* edg) -> int {
    if (g.nseg == 1) {  // plain CSR
      if (off) {
        TRY_CUDA_ST(cudaMemcpyAsync(rel.data(), doff, 4 * entries, cudaMemcpyDeviceToHost, s));
        TRY_CUDA_ST(cudaStreamSynchronize(s));
        for (uint64_t v = 0; v < entries; ++v) off[v] = rel[v];
      }
      if (edg && g.m) TRY_CUDA_ST(cudaMemcpyAsync(edg, dedg, 4 * g.m, cudaMemcpyDeviceToHost, s));
      return PRX_OK;
    }
    TRY_CUDA_ST(cudaMemcpyAsync(rel.data(), doff, 4 * entries, cudaMemcpyDeviceToHost, s));
    TRY_CUDA_ST(cudaStreamSynchronize(s));
    const uint32_t S = g.seg_shift;
    for (uint32_t k = 0; k < g.nseg; ++k) {
      const uint64_t v0 = (uint64_t)k << S, v1 = std::min<uint64_t>(g.n, v0 + (1ull << S));
      for (uint64_t v = v0; v <= v1; ++v) {
        const uint64_t o = seg0[k] + rel[v + k];
        if (off) off[v] = o;
        if (v == v1 && edg && o > seg0[k])
          TRY_CUDA_ST(cudaMemcpyAsync(edg + seg0[k], dedg + pos[k], 4 * (o - seg0[k]), cudaMemcpyDeviceToHost, s));
      }
    }
    return PRX_OK;
  };
  int st = PRX_OK;
  if (xoff || xedg) st = one(g.xoff, g.xedg, g.xseg0, g.xpos, xoff, xedg);
  if (st == PRX_OK && (xtoff || xtedg)) st = one(g.xtoff, g.xtedg, g.xtseg0, g.xtpos, xtoff, xtedg);
  if (st) return st;
  if (xtdat && g.n) TRY_CUDA_ST(cudaMemcpyAsync(xtdat, g.xtdat, 4 * (size_t)g.n, cudaMemcpyDeviceToHost, s));
  TRY_CUDA_ST(cudaStreamSynchronize(s));
  return PRX_OK;
}

int prx_graph_destroy(prx_graph* gr) {
  // Does not touch the context, which may already be destroyed: cudaFree
  // waits for the device's outstanding work on these arrays.
  if (!gr) return PRX_OK;
  cudaSetDevice(gr->g.device);
  GraphDev& g = gr->g;
  graph_free({g.xoff, g.xedg, g.xtoff, g.xtedg, g.xtdat, g.cls_list, g.xbase, g.xtbase, g.low_bm, g.rcp, g.rcp32});
  drop_weights(g);
  cudaFree(g.ocls_list);
  free_chunks(g);
  free_hot(g);
  delete gr;
  return PRX_OK;
}

int prx_graph_size(const prx_graph* gr, uint32_t* n, uint64_t* m) {
  if (!gr) FAIL(PRX_EINVAL, "prx_graph_size: NULL graph");
  if (n) *n = gr->g.n;
  if (m) *m = gr->g.m;
  return PRX_OK;
}

int prx_graph_class_stats(const prx_graph* gr, uint32_t vertices[3], uint64_t edges[3]) {
  if (!gr) FAIL(PRX_EINVAL, "prx_graph_class_stats: NULL graph");
  for (int k = 0; k < NCLS; ++k) {
    if (vertices) vertices[k] = gr->g.cls_begin[k + 1] - gr->g.cls_begin[k];
    if (edges) edges[k] = gr->g.cls_edges[k];
  }
  return PRX_OK;
}

int prx_graph_download(prx_graph* gr, uint32_t* xoff, uint32_t* xedg, uint32_t* xtoff, uint32_t* xtedg,
                       uint32_t* xtdat) {
  if (!gr) FAIL(PRX_EINVAL, "prx_graph_download: NULL graph");
  const GraphDev& g = gr->g;
  cudaStream_t s = gr->ctx->stream;
  TRY_CUDA_ST(cudaSetDevice(gr->ctx->device));
  if ((xoff || xedg) && !g.xoff) FAIL(PRX_ESTATE, "prx_graph_download: graph has no out-CSR");
  if (g.nseg > 1) {  // row segments: rebuild the offsets, 32-bit when they fit
    if (g.m >= 0xffffffffull) FAIL(PRX_ERANGE, "prx_graph_download: 2^32 edges or more; use prx_graph_download64");
    std::vector<uint64_t> o((xoff ? (size_t)g.n + 1 : 0)), ot((xtoff ? (size_t)g.n + 1 : 0));
    const int st = prx_graph_download64(gr, xoff ? o.data() : nullptr, xedg, xtoff ? ot.data() : nullptr, xtedg,
                                        xtdat);
    if (st) return st;
    for (size_t v = 0; v < o.size(); ++v) xoff[v] = (uint32_t)o[v];
    for (size_t v = 0; v < ot.size(); ++v) xtoff[v] = (uint32_t)ot[v];
    return PRX_OK;
  }
  if (xoff) TRY_CUDA_ST(cudaMemcpyAsync(xoff, g.xoff, 4 * ((size_t)g.n + 1), cudaMemcpyDeviceToHost, s));
  if (xedg && g.m) TRY_CUDA_ST(cudaMemcpyAsync(xedg, g.xedg, 4 * g.m, cudaMemcpyDeviceToHost, s));
  if (xtoff) TRY_CUDA_ST(cudaMemcpyAsync(xtoff, g.xtoff, 4 * ((size_t)g.n + 1), cudaMemcpyDeviceToHost, s));
  if (xtedg && g.m) TRY_CUDA_ST(cudaMemcpyAsync(xtedg, g.xtedg, 4 * g.m, cudaMemcpyDeviceToHost, s));
  if (xtdat && g.n) TRY_CUDA_ST(cudaMemcpyAsync(xtdat, g.xtdat, 4 * (size_t)g.n, cudaMemcpyDeviceToHost, s));
  TRY_CUDA_ST(cudaStreamSynchronize(s));
  return PRX_OK;
}

int prx_graph_apply_batch(prx_graph* gr, const uint32_t* du, const uint32_t* dv, uint64_t nd, const uint32_t* iu,
                          const uint32_t* iv, uint64_t ni) {
  if (!gr) FAIL(PRX_EINVAL, "prx_graph_apply_batch: NULL graph");
  GraphDev& g = gr->g;
  prx_context* c = gr->ctx;
  if (!g.xoff) FAIL(PRX_ESTATE, "prx_graph_apply_batch: graph has no out-CSR");
  if (ni && !iv) FAIL(PRX_EINVAL, "prx_graph_apply_batch: insertions need targets");
  int st = check_batch_ids(g.n, du, dv, nd, iu, iv, ni);
  if (st) return st;
  auto sorted_unique = [](const uint32_t* a, const uint32_t* b, uint64_t len) {
    for (uint64_t i = 1; i < len; ++i)
      if (a[i - 1] > a[i] || (a[i - 1] == a[i] && b[i - 1] >= b[i])) return false;
    return true;
  };
  if (!sorted_unique(du, dv, nd) || !sorted_unique(iu, iv, ni))
    FAIL(PRX_EINVAL, "prx_graph_apply_batch: batch must be sorted by (u, v) and unique (tidyBatchUpdateU)");
  if (g.nseg == 1 && g.m - nd + ni > 0xffffffffull)
    FAIL(PRX_ERANGE, "prx_graph_apply_batch: edge count would reach 2^32 (create the graph with prx_graph_create64)");
  if (nd + ni > kMaxVertices) FAIL(PRX_ERANGE, "prx_graph_apply_batch: batch too large");
  // The in-CSR wants the batch ordered by (v, u): the device sorts copies of
  // the (u, v)-sorted lists by v (batch_by_target).
  TRY_CUDA_ST(cudaSetDevice(c->device));
  st = ensure_batch(c, 4 * (size_t)(nd + ni));
  if (st) return st;
  uint32_t* b = c->batch;
  if (nd) TRY_CUDA_ST(cudaMemcpyAsync(b, du, 4 * nd, cudaMemcpyHostToDevice, c->stream));
  if (nd) TRY_CUDA_ST(cudaMemcpyAsync(b + nd, dv, 4 * nd, cudaMemcpyHostToDevice, c->stream));
  if (ni) TRY_CUDA_ST(cudaMemcpyAsync(b + 2 * nd, iu, 4 * ni, cudaMemcpyHostToDevice, c->stream));
  if (ni) TRY_CUDA_ST(cudaMemcpyAsync(b + 2 * nd + ni, iv, 4 * ni, cudaMemcpyHostToDevice, c->stream));
  uint32_t* t = b + 2 * (nd + ni);
  TRY_CUDA_ST(batch_by_target(b, b + nd, (uint32_t)nd, g.n, t, t + nd, c->sms, c->stream));
  TRY_CUDA_ST(batch_by_target(b + 2 * nd, b + 2 * nd + ni, (uint32_t)ni, g.n, t + 2 * nd, t + 2 * nd + ni, c->sms,
                              c->stream));
  const cudaError_t e = apply_batch_device(g, c->batch, nd, ni, c->sms, c->stream);
  if (e == cudaErrorInvalidValue)
    FAIL(PRX_EINVAL, "prx_graph_apply_batch: batch is not tidy (a deletion is missing or an insertion exists)");
  if (e == cudaErrorInvalidConfiguration)
    FAIL(PRX_ERANGE, "prx_graph_apply_batch: a row segment would hold 2^32 edges or more");
  TRY_CUDA_ST(e);
  drop_weights(g);  // the edges changed: weights must be set again
  return PRX_OK;
}

// Sets the L2 fetch granularity hint for the life of a solve and puts the
// process's previous setting back afterwards (bytes <= 0: leaves it).
struct FetchGuard {
  size_t prev = 0;
  bool set = false;
  explicit FetchGuard(int bytes) {
    if (bytes <= 0 || cudaDeviceGetLimit(&prev, cudaLimitMaxL2FetchGranularity) != cudaSuccess) return;
    if (prev != (size_t)bytes) set = cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)bytes) == cudaSuccess;
  }
  ~FetchGuard() {
    if (set) cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, prev);
  }
};

static int solve_common(prx_context* c, prx_graph* gr, int mode, const uint32_t* du, const uint32_t* dv,
                        uint64_t nd, const uint32_t* iu, const uint32_t* iv, uint64_t ni, const double* q,
                        const prx_options* o, double* ranks_out, prx_result* res, bool host) {
  if (!c || !gr || gr->ctx != c) FAIL(PRX_EINVAL, "prx_solve: bad context or graph");
  if (!valid_mode(mode)) FAIL(PRX_EINVAL, "prx_solve: unknown mode");
  prx_options opt;
  prx_options_default(&opt);
  if (o) opt = *o;
  if (!(opt.damping > 0 && opt.damping < 1)) FAIL(PRX_EINVAL, "prx_solve: damping must be in (0, 1)");
  if (opt.l2_fetch_bytes < -1 || opt.l2_fetch_bytes > 128)
    FAIL(PRX_EINVAL, "prx_solve: l2_fetch_bytes must be in -1 .. 128");
  if (opt.hot_sources < -1) FAIL(PRX_EINVAL, "prx_solve: hot_sources must be -1, 0 or a vertex count");
  if (opt.int_adds < -1 || opt.int_adds > 4) FAIL(PRX_EINVAL, "prx_solve: int_adds must be in -1 .. 4");
  if (!ranks_out && gr->g.n) FAIL(PRX_EINVAL, "prx_solve: ranks_out is NULL");
  prx_result own;
  if (!res) res = &own;  // the convergence check reads it
  std::memset(res, 0, sizeof(*res));
  const GraphDev& g = gr->g;
  if (g.n == 0) return PRX_OK;  // empty graph: the reference returns {} (:869)
  const bool dyn = mode >= PRX_DYNAMIC_TRAVERSAL;
  if (!dyn) nd = ni = 0;
  TRY_CUDA_ST(cudaSetDevice(c->device));
  const uint32_t *ddu = du, *ddv = dv, *diu = iu;
  const double* dq = q;
  int st;
  if (host) {
    if (dyn) {
      st = check_batch_ids(g.n, du, dv, nd, iu, iv, ni);
      if (st) return st;
      st = ensure_batch(c, 2 * nd + ni);
      if (st) return st;
      if (nd) {
        TRY_CUDA_ST(cudaMemcpyAsync(c->batch, du, 4 * nd, cudaMemcpyHostToDevice, c->stream));
        TRY_CUDA_ST(cudaMemcpyAsync(c->batch + nd, dv, 4 * nd, cudaMemcpyHostToDevice, c->stream));
      }
      if (ni) TRY_CUDA_ST(cudaMemcpyAsync(c->batch + 2 * nd, iu, 4 * ni, cudaMemcpyHostToDevice, c->stream));
      ddu = c->batch; ddv = c->batch + nd; diu = c->batch + 2 * nd;
    }
    st = ensure_ws(c, g.n, dyn);
    if (st) return st;
    if (q && mode != PRX_STATIC) {
      // stage q in r[1]: init reads it before anything writes r[1]
      TRY_CUDA_ST(cudaMemcpyAsync(c->r[1], q, sizeof(double) * g.n, cudaMemcpyHostToDevice, c->stream));
      dq = c->r[1];
    } else {
      dq = nullptr;
    }
  }
  const double* fr = nullptr;
  // held until the stream is drained below (the destructor runs after it)
  FetchGuard fetch(opt.l2_fetch_bytes == 0 ? g.tuned_fetch : opt.l2_fetch_bytes);
  st = solve_core(c, gr, mode, ddu, ddv, nd, diu, ni, dq, opt, res, &fr);
  if (st) {
    cudaStreamSynchronize(c->stream);
    return st;
  }
  TRY_CUDA_ST(cudaMemcpyAsync(ranks_out, fr, sizeof(double) * g.n,
                              host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, c->stream));
  TRY_CUDA_ST(cudaStreamSynchronize(c->stream));
  if (opt.require_convergence && !(res->last_delta < opt.tolerance))
    FAIL(PRX_ENOCONV, "prx_solve: the iteration cap was reached before the L-inf test passed");
  return PRX_OK;
}

int prx_solve(prx_context* c, prx_graph* gr, int mode, const uint32_t* du, const uint32_t* dv, uint64_t nd,
              const uint32_t* iu, const uint32_t* iv, uint64_t ni, const double* q, const prx_options* o,
              double* ranks_out, prx_result* res) {
  return solve_common(c, gr, mode, du, dv, nd, iu, iv, ni, q, o, ranks_out, res, true);
}

int prx_solve_device(prx_context* c, prx_graph* gr, int mode, const uint32_t* du, const uint32_t* dv, uint64_t nd,
                     const uint32_t* iu, const uint32_t* iv, uint64_t ni, const double* q, const prx_options* o,
                     double* ranks_out, prx_result* res) {
  return solve_common(c, gr, mode, du, dv, nd, iu, iv, ni, q, o, ranks_out, res, false);
}

int prx_selftest_division(prx_context* c, uint32_t dmax, uint32_t per, unsigned long long* mismatches) {
  if (!c || !mismatches) FAIL(PRX_EINVAL, "prx_selftest_division: bad context or NULL output");
  if (dmax == 0 || per == 0) FAIL(PRX_EINVAL, "prx_selftest_division: dmax and per must be positive");
  TRY_CUDA_ST(cudaSetDevice(c->device));
  TRY_CUDA_ST(selftest_division(dmax, per, mismatches, c->sms, c->stream));
  return PRX_OK;
}

int prx_mark_affected(prx_context* c, prx_graph* gr, int mode, const uint32_t* du, const uint32_t* dv, uint64_t nd,
                      const uint32_t* iu, uint64_t ni, uint8_t* flags_out) {
  if (!c || !gr || gr->ctx != c) FAIL(PRX_EINVAL, "prx_mark_affected: bad context or graph");
  if (mode < PRX_DYNAMIC_TRAVERSAL || mode > PRX_PRUNE_DYNAMIC_FRONTIER)
    FAIL(PRX_EINVAL, "prx_mark_affected: mode must be DT, DF or DF-P");
  const GraphDev& g = gr->g;
  if (!g.xoff) FAIL(PRX_ESTATE, "prx_mark_affected: graph has no out-CSR");
  if (g.n == 0) return PRX_OK;
  if (!flags_out) FAIL(PRX_EINVAL, "prx_mark_affected: flags_out is NULL");
  int st = check_batch_ids(g.n, du, dv, nd, iu, nullptr, ni);
  if (st) return st;
  TRY_CUDA_ST(cudaSetDevice(c->device));
  st = ensure_ws(c, g.n, true);
  if (st) return st;
  st = ensure_batch(c, 2 * nd + ni);
  if (st) return st;
  cudaStream_t s = c->stream;
  if (nd) {
    TRY_CUDA_ST(cudaMemcpyAsync(c->batch, du, 4 * nd, cudaMemcpyHostToDevice, s));
    TRY_CUDA_ST(cudaMemcpyAsync(c->batch + nd, dv, 4 * nd, cudaMemcpyHostToDevice, s));
  }
  if (ni) TRY_CUDA_ST(cudaMemcpyAsync(c->batch + 2 * nd, iu, 4 * ni, cudaMemcpyHostToDevice, s));
  prx_options o;
  prx_options_default(&o);
  const SolveArgs a = make_args(c, g, o);
  launch_state_reset(c->st, 0, 0.0, s);
  st = run_marking(c, a, mode, c->batch, c->batch + nd, nd, c->batch + 2 * nd, ni);
  if (st) return st;
  launch_flags_from_bitmap(c->bm[0], c->flags, g.n, s);
  TRY_CUDA_ST(cudaMemcpyAsync(flags_out, c->flags, g.n, cudaMemcpyDeviceToHost, s));
  TRY_CUDA_ST(cudaStreamSynchronize(s));
  TRY_CUDA_ST(cudaGetLastError());
  return PRX_OK;
}

}  // extern "C"
