// prx_ctx.h -- the opaque handles of the C ABI (contexts and device graphs)
// and the status macros shared by the host drivers.  Internal.
#pragma once
#include <string>
#include <vector>
#include "prx_internal.h"

namespace prx {
struct PprWs;
void ppr_free(PprWs* w);  // prx_ppr.cu
}  // namespace prx

using namespace prx;

struct prx_context {
  int device = 0;
  int sms = 152;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // graph uploads overlapped with layout builds (created on first use)
  State* st = nullptr;        // device control block
  State* st_host = nullptr;   // pinned: [0] after marking, [1] loop checks
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // workspace (grows on demand)
  uint32_t ws_n = 0;
  bool ws_dyn = false;
  double* r[2] = {nullptr, nullptr};
  double* c[2] = {nullptr, nullptr};
  double* acc64 = nullptr;    // partial sums between chunk passes
  double* ch[2] = {nullptr, nullptr};  // dense copies of the hot sources' contributions
  uint32_t ch_n = 0;
  float* acc32 = nullptr;
  uint8_t* flags = nullptr;   // byte flags for prx_mark_affected
  uint32_t* bm[3] = {nullptr, nullptr, nullptr};
  uint32_t* nf[2] = {nullptr, nullptr};
  uint32_t* xb = nullptr;
  uint32_t* naff = nullptr;
  uint32_t* ever = nullptr;   // FP32 dynamic phase: vertices updated at least once
  double* pf = nullptr;       // DF-P: 1 / (1 - P/d) per vertex
  uint32_t* lists[2][NCLS] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  uint32_t* xl = nullptr;
  uint32_t* fr[3] = {nullptr, nullptr, nullptr};
  // FP32 refinement (grown on first use)
  uint32_t ws32_n = 0;
  float* rho = nullptr;
  float* e32[2] = {nullptr, nullptr};
  float* ce32[2] = {nullptr, nullptr};
  uint32_t* batch = nullptr;  // device copy of a batch
  size_t batch_cap = 0;       // in uint32 elements
  // launch accounting and optional per-launch timing of the rank update
  uint64_t launches = 0;
  std::vector<cudaEvent_t> tev;   // pairs: start, end
  std::vector<int> tev_cls;       // class of each recorded pair
  size_t tev_used = 0;            // pairs recorded since the last drain
  double upd_ms[2 * NCLS] = {0, 0, 0, 0, 0, 0};     // [FP64 classes | FP32 classes]
  uint32_t upd_n[2 * NCLS] = {0, 0, 0, 0, 0, 0};
  prx::PprWs* ppr = nullptr;  // batched personalized PageRank workspace (prx_ppr.cu)
  double* wk = nullptr;       // weighted solves and the adjoint: 3 n-vectors + partial sums (prx_weighted.cu)
  size_t wk_cap = 0;          // in doubles
};

struct prx_graph {
  prx_context* ctx = nullptr;
  GraphDev g;
};

// Solve pieces shared by prx_solve and the multi-batch solve (prx_api.cu).
int ensure_ws(prx_context* c, uint32_t n, bool dyn);
// The dense hot-source copies c->ch[2] for hot_n sources.
int ensure_ch(prx_context* c, uint32_t hot_n);
SolveArgs make_args(prx_context* c, const GraphDev& g, const prx_options& o);
// DF / DF-P marking runs without host synchronisation; DT's closure reads
// the control block.
int run_marking(prx_context* c, const SolveArgs& a, int mode, const uint32_t* du, const uint32_t* dv, uint64_t nd,
                const uint32_t* iu, uint64_t ni);
// One iteration (update launches, expansion, k_finalize) on stream c->stream.
int enqueue_iteration(prx_context* c, const GraphDev& g, const SolveArgs& a, int mode, bool timing,
                      const ChunkLayout* lay);
// Keeps a conditional WHILE node going while the solve is not done and fewer
// than cap bodies ran (counted in st->graph_rounds).
__global__ void k_loop_cond(cudaGraphConditionalHandle h, State* st, int cap);

namespace prx {
// Inside a capture on s: a conditional node of `type` whose handle (default
// dflt) is set by `arm` launched on s just before the node, and whose body is
// captured on s2 by body(s2).  Leaves s depending on the node.
template <class Arm, class Body>
inline cudaError_t capture_conditional(cudaStream_t s, cudaStream_t s2, cudaGraphConditionalNodeType type,
                                       unsigned dflt, Arm arm, Body body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr);
  cudaGraphConditionalHandle h{};
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, dflt, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return e;
  arm(h);
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edata = nullptr;
  size_t ndeps = 0;
  e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, &edata, &ndeps);
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = type;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, deps, edata, ndeps, &p);
  if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(s2, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  const cudaError_t eb = body(s2, h);
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(s2, &captured);  // always leave capture mode
  return eb != cudaSuccess ? eb : e;
}

}  // namespace prx

#define TRY_CUDA_ST(x)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (x);                                                                \
    if (e_ != cudaSuccess) {                                                             \
      set_error(std::string(#x) + ": " + cudaGetErrorString(e_));                        \
      return e_ == cudaErrorMemoryAllocation ? PRX_ENOMEM : PRX_ECUDA;                   \
    }                                                                                    \
  } while (0)

#define FAIL(code, msg)  \
  do {                   \
    set_error(msg);      \
    return (code);       \
  } while (0)

