// prx_multibatch.cu -- K consecutive batch updates, each applied to the graph
// and followed by a DF or DF-P solve, as ONE CUDA graph launch.
//
// The reference's driver runs its batches one after another: apply batch k
// to the graph (on the host, applyBatchUpdateOmpU, inc/batch.hxx:239-247),
// transpose, then solve from the previous ranks (main.cu:88-147, the
// dynamic calls at :113-123).  Here the whole sequence is one graph:
//
//   step k:  gate (no error so far) -> IF { tidiness check of batch k }
//            gate (no error so far) -> IF { apply batch k into the other of
//              two ping-pong CSR sets; LOW bitmap and reciprocals of the new
//              version; state reset; ranks from the previous step; marking;
//              WHILE { one iteration } ; record step k }
//
// Every count stays on the device (apply_batch_graph), the iteration loop is
// the conditional WHILE node of the single-solve graph loop, and the batch
// lists' (v, u) orders are sorted before the launch.  A batch that is not
// tidy stops the sequence: later steps' gates stay closed, the graph keeps
// the batches before it, and the call reports which step failed.
//
// Each step gathers like a single solve does: its LOW rows regrouped by
// source chunk (rebuilt by kernels for the step's graph version) with the
// edges from hot sources read from their dense copy.  The hot set is the one
// of the graph before the batches: any set of sources gives the same sums
// (the copy holds the same values), and a few batches barely move the
// out-degree ranking.
#include <algorithm>
#include <cstring>
#include <vector>
#include "prx_ctx.h"
#include "prx_device.cuh"

namespace prx {

struct MbRecord {
  int iterations;
  uint32_t pad;
  unsigned long long affected;
  unsigned long long edges;
  double last_delta;
  // %globaltimer after the step's initialisation (apply, vertex tables,
  // layout, ranks), after its marking, and at its end
  unsigned long long t_init_ns, t_mark_ns, t_ns;
};

struct MbControl {
  uint32_t err;      // batch check (launch_batch_check's bits)
  uint32_t applied;  // steps completed
  unsigned long long t0_ns;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void k_mb_start(MbControl* m) {
  m->err = 0;
  m->applied = 0;
  m->t0_ns = global_ns();
}

__global__ void k_mb_stamp(unsigned long long* t) { *t = global_ns(); }

__global__ void k_mb_gate(cudaGraphConditionalHandle h, const MbControl* m) {
  cudaGraphSetConditional(h, m->err == 0 ? 1u : 0u);
}

// Step k's ranks (parity iter & 1) become the next step's start (qbuf) and,
// with each, row k of the per-step output; thread 0 records the step.
__global__ void k_mb_record(const State* st, const double* r0, const double* r1, double* qbuf, double* each,
                            uint32_t n, MbRecord* rec, MbControl* m, uint32_t step) {
  const double* r = (st->iter & 1) ? r1 : r0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const double x = r[v];
    qbuf[v] = x;
    if (each) each[v] = x;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    rec->iterations = st->iter;
    rec->affected = st->affected;
    rec->edges = st->edges;
    rec->last_delta = st->last_delta;
    rec->t_ns = global_ns();
    m->applied = step + 1;
  }
}

}  // namespace prx

using namespace prx;

extern "C" int prx_solve_batches_device(prx_context* c, prx_graph* gr, int mode, uint32_t K, const uint64_t* del_off,
                                        const uint32_t* del_u, const uint32_t* del_v, const uint64_t* ins_off,
                                        const uint32_t* ins_u, const uint32_t* ins_v, const double* q,
                                        const prx_options* o, double* ranks_out, double* ranks_each,
                                        prx_result* res, uint32_t* applied_out) {
  if (applied_out) *applied_out = 0;
  if (!c || !gr || gr->ctx != c) FAIL(PRX_EINVAL, "prx_solve_batches_device: bad context or graph");
  GraphDev& g = gr->g;
  if (mode != PRX_DYNAMIC_FRONTIER && mode != PRX_PRUNE_DYNAMIC_FRONTIER)
    FAIL(PRX_EINVAL, "prx_solve_batches_device: DF and DF-P only");
  if (!g.xoff) FAIL(PRX_ESTATE, "prx_solve_batches_device: the graph needs its out-CSR");
  if (g.nseg > 1) FAIL(PRX_ERANGE, "prx_solve_batches_device: not for graphs with row segments (64-bit offsets)");
  if (!q || !ranks_out || (K && (!del_off || !ins_off))) FAIL(PRX_EINVAL, "prx_solve_batches_device: NULL argument");
  prx_options opt;
  prx_options_default(&opt);
  if (o) opt = *o;
  if (opt.precision != PRX_FP64) FAIL(PRX_EINVAL, "prx_solve_batches_device: FP64 only");
  if (!(opt.damping > 0 && opt.damping < 1)) FAIL(PRX_EINVAL, "prx_solve_batches_device: damping must be in (0, 1)");
  if (opt.int_adds < -1 || opt.int_adds > 4) FAIL(PRX_EINVAL, "prx_solve_batches_device: int_adds must be in -1 .. 4");
  const uint32_t n = g.n;
  TRY_CUDA_ST(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  if (K == 0) {
    TRY_CUDA_ST(cudaMemcpyAsync(ranks_out, q, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    TRY_CUDA_ST(cudaStreamSynchronize(s));
    return PRX_OK;
  }
  // edge counts along the sequence (tidy batches) and the largest batch
  std::vector<uint64_t> m(K + 1);
  m[0] = g.m;
  uint64_t cap = g.m, bmax = 1, btotal = 0;
  for (uint32_t k = 0; k < K; ++k) {
    if (del_off[k + 1] < del_off[k] || ins_off[k + 1] < ins_off[k])
      FAIL(PRX_EINVAL, "prx_solve_batches_device: batch offsets must not decrease");
    const uint64_t nd = del_off[k + 1] - del_off[k], ni = ins_off[k + 1] - ins_off[k];
    if (nd > m[k]) FAIL(PRX_EINVAL, "prx_solve_batches_device: more deletions than edges");
    if ((nd && (!del_u || !del_v)) || (ni && (!ins_u || !ins_v)))
      FAIL(PRX_EINVAL, "prx_solve_batches_device: NULL batch array");
    m[k + 1] = m[k] - nd + ni;
    cap = std::max(cap, m[k + 1]);
    bmax = std::max(bmax, nd + ni);
    btotal += nd + ni;
  }
  if (cap > 0xfffffff0ull || bmax > kMaxVertices)
    FAIL(PRX_ERANGE, "prx_solve_batches_device: 2^32 edges or more (use prx_graph_create64 and single batches)");
  int st = ensure_ws(c, n, true);
  if (st) return st;

  // device buffers: two CSR sets with their vertex tables, the batches with
  // their (v, u) orders, the apply workspace, the carried ranks and records
  // (from the graph pool: the set that ends up holding the graph stays)
  std::vector<void*> owned;
  auto alloc = [&](void** p, size_t bytes) -> cudaError_t {
    const cudaError_t e = graph_alloc(p, bytes ? bytes : 4, s);
    if (e == cudaSuccess) owned.push_back(*p);
    return e;
  };
  auto release = [&]() {
    for (void* p : owned) cudaFreeAsync(p, s);
    owned.clear();
    cudaStreamSynchronize(s);
  };
#define MB_TRY(x)                                                                    \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) {                                                         \
      release();                                                                     \
      set_error(std::string("prx_solve_batches_device: ") + cudaGetErrorString(e_)); \
      return e_ == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;               \
    }                                                                                \
  } while (0)
  const size_t words = ((size_t)n + 31) / 32;
  CsrSet set[2];
  uint32_t* low[2];
  double* rcp[2];
  float* rcp32[2];
  for (int i = 0; i < 2; ++i) {
    MB_TRY(alloc((void**)&set[i].xoff, 4 * ((size_t)n + 1)));
    MB_TRY(alloc((void**)&set[i].xtoff, 4 * ((size_t)n + 1)));
    MB_TRY(alloc((void**)&set[i].xedg, 4 * cap));
    MB_TRY(alloc((void**)&set[i].xtedg, 4 * edge_slots(cap)));
    MB_TRY(alloc((void**)&set[i].xtdat, 4 * (size_t)n));
    MB_TRY(alloc((void**)&low[i], 4 * (words + 1)));
    MB_TRY(alloc((void**)&rcp[i], 8 * (size_t)n));
    MB_TRY(alloc((void**)&rcp32[i], 4 * (size_t)n));
  }
  uint32_t* bat = nullptr;   // per batch: [du | dv | iu | iv | tdk | tdv | tik | tiv]
  MB_TRY(alloc((void**)&bat, 4 * 4 * btotal));
  std::vector<size_t> bpos(K + 1, 0);
  for (uint32_t k = 0; k < K; ++k) {
    const uint64_t nd = del_off[k + 1] - del_off[k], ni = ins_off[k + 1] - ins_off[k];
    uint32_t* b = bat + bpos[k];
    bpos[k + 1] = bpos[k] + 4 * (nd + ni);
    if (nd) {
      MB_TRY(cudaMemcpyAsync(b, del_u + del_off[k], 4 * nd, cudaMemcpyDeviceToDevice, s));
      MB_TRY(cudaMemcpyAsync(b + nd, del_v + del_off[k], 4 * nd, cudaMemcpyDeviceToDevice, s));
    }
    if (ni) {
      MB_TRY(cudaMemcpyAsync(b + 2 * nd, ins_u + ins_off[k], 4 * ni, cudaMemcpyDeviceToDevice, s));
      MB_TRY(cudaMemcpyAsync(b + 2 * nd + ni, ins_v + ins_off[k], 4 * ni, cudaMemcpyDeviceToDevice, s));
    }
    uint32_t* t = b + 2 * (nd + ni);
    MB_TRY(batch_by_target(b, b + nd, (uint32_t)nd, n, t, t + nd, c->sms, s));
    MB_TRY(batch_by_target(b + 2 * nd, b + 2 * nd + ni, (uint32_t)ni, n, t + 2 * nd, t + 2 * nd + ni, c->sms, s));
  }
  // the steps' LOW layout: source chunks as a single solve picks them, hot
  // sources of the graph before the batches
  const bool hot = opt.hot_sources >= 0;
  if (hot) {
    MB_TRY(ensure_hot(g, opt.hot_sources > 0 ? (uint32_t)opt.hot_sources : kDefaultHotCap, c->sms, s));
    if (g.hot_n && (st = ensure_ch(c, g.hot_n))) {
      release();
      return st;
    }
  }
  const uint32_t width = opt.chunk_vertices ? opt.chunk_vertices : g.tuned_w64 ? g.tuned_w64 : kDefaultChunk64;
  const int KC = (int)std::max<uint64_t>(1, ((uint64_t)n + width - 1) / width);
  const bool use_lay = n > 0 && (KC > 1 || (hot && g.hot_n > 0)) && (uint64_t)KC * ((uint64_t)n + 1) < 0xffffffffull;
  // two layout buffers: step k >= 1 carries step k-1's layout to its version
  uint32_t *lay_off[2] = {nullptr, nullptr}, *lay_edg[2] = {nullptr, nullptr}, *lay_ws = nullptr;
  if (use_lay) {
    const uint32_t len = (uint32_t)((uint64_t)KC * ((uint64_t)n + 1));
    for (int i = 0; i < 2; ++i) {
      MB_TRY(alloc((void**)&lay_off[i], 4 * (size_t)len));
      MB_TRY(alloc((void**)&lay_edg[i], 4 * edge_slots(cap)));
    }
    MB_TRY(alloc((void**)&lay_ws, 4 * (size_t)scan_ws_words(len)));
  }
  uint32_t* wsbuf = nullptr;
  MB_TRY(alloc((void**)&wsbuf, 4 * ApplyWs::words(n, (uint32_t)bmax)));
  const ApplyWs ws(wsbuf, n, (uint32_t)bmax);
  double* qbuf = nullptr;
  MB_TRY(alloc((void**)&qbuf, 8 * (size_t)n));
  MB_TRY(cudaMemcpyAsync(qbuf, q, 8 * (size_t)n, cudaMemcpyDeviceToDevice, s));
  MbRecord* rec = nullptr;
  MbControl* ctl = nullptr;
  MB_TRY(alloc((void**)&rec, sizeof(MbRecord) * K));
  MB_TRY(alloc((void**)&ctl, sizeof(MbControl)));
  MB_TRY(cudaStreamSynchronize(s));

  // the sequence as one graph
  const CsrSet orig{g.xoff, g.xedg, g.xtoff, g.xtedg, g.xtdat};
  cudaStream_t s2 = nullptr, s3 = nullptr;
  MB_TRY(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamCreateWithFlags(&s3, cudaStreamNonBlocking);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const int cap_iter = (opt.max_iterations < (1 << 30) ? opt.max_iterations : (1 << 30)) + 2;
  const uint64_t l_start = c->launches;
  uint64_t per_step_fixed = 0, per_body = 0;
  if (e == cudaSuccess) e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t ec = cudaSuccess;
    k_mb_start<<<1, 1, 0, s>>>(ctl);
    for (uint32_t k = 0; k < K && ec == cudaSuccess; ++k) {
      const CsrSet& src = k == 0 ? orig : set[(k - 1) & 1];
      const CsrSet& dst = set[k & 1];
      const uint32_t nd = (uint32_t)(del_off[k + 1] - del_off[k]), ni = (uint32_t)(ins_off[k + 1] - ins_off[k]);
      const uint32_t* b = bat + bpos[k];
      auto gate = [&](cudaGraphConditionalHandle h) { k_mb_gate<<<1, 1, 0, s>>>(h, ctl); };
      ec = capture_conditional(s, s2, cudaGraphCondTypeIf, 0, gate, [&](cudaStream_t sb, cudaGraphConditionalHandle) {
        launch_batch_check(src.xoff, src.xedg, n, b, nd, ni, &ctl->err, c->sms, sb);
        return cudaGetLastError();
      });
      if (ec != cudaSuccess) break;
      ec = capture_conditional(s, s2, cudaGraphCondTypeIf, 0, gate, [&](cudaStream_t sb, cudaGraphConditionalHandle) {
        cudaError_t eb = apply_batch_graph(src, dst, n, b, nd, ni, ws, c->sms, sb);
        if (eb != cudaSuccess) return eb;
        launch_vertex_tables(dst.xtoff, 32, dst.xtdat, n, low[k & 1], rcp[k & 1], rcp32[k & 1], c->sms, sb);
        ChunkLayout lay;
        if (use_lay) {
          lay.width = width;
          lay.K = KC;
          lay.hot = hot && g.hot_n > 0;
          lay.off = lay_off[k & 1];
          lay.edg = lay_edg[k & 1];
          if (k == 0) {
            eb = build_layout_into(dst.xtoff, dst.xtedg, low[0], n, width, KC, lay.hot ? g.hot_idx : nullptr,
                                   (n + 31) / 32, lay.off, lay.edg, lay_ws, c->sms, sb);
          } else {  // the in-CSR's touched rows of this apply: its bitmap, list and count in ws
            ChunkLayout prev = lay;
            prev.off = lay_off[(k - 1) & 1];
            prev.edg = lay_edg[(k - 1) & 1];
            const uint32_t words32 = (n + 31) / 32;
            eb = carry_layout(prev, dst.xtoff, dst.xtedg, n, ws.touched + words32, ws.trow, 0, ws.cnt + words32,
                              g.hot_idx, lay.off, lay.edg, lay_ws, c->sms, sb);
            prev.off = prev.edg = nullptr;  // owned by the buffers above
          }
          if (eb != cudaSuccess) return eb;
        }
        GraphDev view;  // step k's graph version
        view.n = n;
        view.m = m[k + 1];
        view.xoff = dst.xoff; view.xedg = dst.xedg;
        view.xtoff = dst.xtoff; view.xtedg = dst.xtedg; view.xtdat = dst.xtdat;
        view.low_bm = low[k & 1];
        view.rcp = rcp[k & 1];
        view.rcp32 = rcp32[k & 1];
        view.mid_max = g.mid_max;
        SolveArgs a = make_args(c, view, opt);
        a.hot_list = g.hot_list;
        a.hot_n = use_lay && lay.hot ? g.hot_n : 0;
        // the solve's launches go to c->stream: point it at the body's stream
        cudaStream_t keep = c->stream;
        c->stream = sb;
        const uint64_t l0 = c->launches;
        launch_state_reset(c->st, opt.max_iterations, opt.tolerance, sb);
        launch_init_ranks(a, qbuf, true, sb);
        launch_hot_copy(a, 0, c->sms, sb);
        if (mode == PRX_PRUNE_DYNAMIC_FRONTIER) launch_prune_factor(a, sb);
        k_mb_stamp<<<1, 1, 0, sb>>>(&rec[k].t_init_ns);
        int sm = run_marking(c, a, mode, b, b + nd, nd, b + 2 * (size_t)nd, ni);
        k_mb_stamp<<<1, 1, 0, sb>>>(&rec[k].t_mark_ns);
        if (!sm) {
          eb = capture_conditional(sb, s3, cudaGraphCondTypeWhile, 1, [](cudaGraphConditionalHandle) {},
                                   [&](cudaStream_t sw, cudaGraphConditionalHandle hw) {
                                     c->stream = sw;
                                     const uint64_t lb = c->launches;
                                     const int si = enqueue_iteration(c, view, a, mode, false,
                                                                      use_lay ? &lay : nullptr);
                                     k_loop_cond<<<1, 1, 0, sw>>>(hw, c->st, cap_iter);
                                     per_body = c->launches - lb + 1;
                                     c->stream = sb;
                                     return si ? cudaErrorUnknown : cudaGetLastError();
                                   });
        }
        c->stream = keep;
        if (sm && eb == cudaSuccess) eb = cudaErrorUnknown;
        if (eb != cudaSuccess) return eb;
        k_mb_record<<<c->sms * 4, 256, 0, sb>>>(c->st, c->r[0], c->r[1], qbuf,
                                                ranks_each ? ranks_each + (size_t)k * n : nullptr, n, rec + k, ctl,
                                                k);
        if (k == 0) per_step_fixed = c->launches - l0 + 3 + (mode == PRX_PRUNE_DYNAMIC_FRONTIER);
        return cudaGetLastError();
      });
    }
    const cudaError_t el = cudaGetLastError();
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(s, &captured);  // always leave capture mode
    graph = captured;
    if (e == cudaSuccess) e = ec;
    if (e == cudaSuccess) e = el;
  }
  c->launches = l_start;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
  std::vector<MbRecord> hrec(K);
  MbControl hctl{};
  if (e == cudaSuccess) e = cudaMemcpyAsync(hrec.data(), rec, sizeof(MbRecord) * K, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hctl, ctl, sizeof(MbControl), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (s2) cudaStreamDestroy(s2);
  if (s3) cudaStreamDestroy(s3);
  MB_TRY(e);

  // the graph becomes the last applied version
  const uint32_t done = hctl.applied;
  if (done > 0) {
    const int keep = (int)((done - 1) & 1);
    graph_free({g.xoff, g.xedg, g.xtoff, g.xtedg, g.xtdat});
    g.xoff = set[keep].xoff; g.xedg = set[keep].xedg;
    g.xtoff = set[keep].xtoff; g.xtedg = set[keep].xtedg; g.xtdat = set[keep].xtdat;
    g.m = g.m_cap = m[done];
    for (void* p : {(void*)set[keep].xoff, (void*)set[keep].xedg, (void*)set[keep].xtoff, (void*)set[keep].xtedg,
                    (void*)set[keep].xtdat})
      owned.erase(std::find(owned.begin(), owned.end(), p));
    drop_weights(g);
    MB_TRY(build_classes(g, c->sms, s));
  }
  MB_TRY(cudaMemcpyAsync(ranks_out, qbuf, 8 * (size_t)n, cudaMemcpyDeviceToDevice, s));
  MB_TRY(cudaStreamSynchronize(s));
  release();
#undef MB_TRY
  if (applied_out) *applied_out = done;
  if (res) {
    unsigned long long t_prev = hctl.t0_ns;
    for (uint32_t k = 0; k < K; ++k) {
      prx_result& r = res[k];
      std::memset(&r, 0, sizeof(r));
      if (k >= done) continue;
      r.iterations = hrec[k].iterations;
      r.time_ms = (float)((hrec[k].t_ns - t_prev) * 1e-6);
      r.initialization_time_ms = (float)((hrec[k].t_init_ns - t_prev) * 1e-6);
      r.marking_time_ms = (float)((hrec[k].t_mark_ns - hrec[k].t_init_ns) * 1e-6);
      r.computation_time_ms = (float)((hrec[k].t_ns - hrec[k].t_mark_ns) * 1e-6);
      t_prev = hrec[k].t_ns;
      r.affected_initial = hrec[k].affected;
      r.edges_processed = hrec[k].edges;
      r.last_delta = hrec[k].last_delta;
      r.kernel_launches = per_step_fixed + per_body * (uint64_t)hrec[k].iterations;
    }
  }
  if (done < K) {
    const char* why = hctl.err & 8   ? " has a vertex id out of range"
                      : hctl.err & 4 ? " has a list not sorted by (u, v) or with repeats"
                      : hctl.err & 1 ? " deletes an edge the graph does not hold"
                                     : " inserts an edge the graph holds";
    set_error("prx_solve_batches_device: batch " + std::to_string(done) + why +
              " (the graph holds the batches before it)");
    return PRX_EINVAL;
  }
  return PRX_OK;
}
