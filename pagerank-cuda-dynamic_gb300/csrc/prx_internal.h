// prx_internal.h -- shared host/device declarations of the GB300 PageRank
// library.  Not part of the public ABI (that is include/pagerank_gb300.h).
#pragma once
#include <cstdint>
#include <cstddef>
#include <initializer_list>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "pagerank_gb300.h"

namespace prx {

// In-degree classes of the pull update.  The 64 boundary is semantic: the
// reference adds the in-edges of a vertex with in-degree <= 64 front to back
// in one thread and those of a vertex with in-degree > 64 in 256 strided
// partial sums folded by a halving tree (inc/pagerankCuda.hxx:93,169,177;
// inc/_cuda.hxx:541-551).  The MID/HIGH boundary only picks warp-per-vertex
// or block-per-vertex execution of that same 256-way order.
constexpr uint32_t kLowMax = 64;
constexpr uint32_t kDefaultMidMax = 4096;
enum Cls { LOW = 0, MID = 1, HIGH = 2, NCLS = 3 };

constexpr int kThreads = 256;  // threads per block for all map-like kernels

// Elements allocated for an in-edge array of m edges: the LOW-class gathers
// read a row's edge ids as aligned 16-byte groups, and the group holding a
// row's last edge may reach 3 ids past the array's end.
inline size_t edge_slots(uint64_t m) { return (size_t)((m + 3) & ~3ull) + 4; }

// Largest vertex count: 2^32 - 2^24, so no 32-bit grid-stride loop index
// (strides stay below 2^24 threads) can wrap past n.
constexpr uint32_t kMaxVertices = 0xFF000000u;

// Device-resident control block of one solve.
struct State {
  unsigned long long el_bits[2];  // L-inf delta of the iteration with parity p (bits of a double >= 0)
  int iter;                       // iterations completed
  int done;                       // set once el < tol or iter == max_iter
  int max_iter;
  int pad0;
  double tol;
  double last_delta;
  uint32_t cnt[2][NCLS];          // dynamic: queued MID / HIGH vertices (cnt[0][MID], cnt[0][HIGH])
  uint32_t xcnt;                  // vertices whose out-neighbours must be marked
  uint32_t fcnt[3];               // DT closure frontier lengths, rotating over levels
  uint32_t pcnt[3];               // DT closure by pull rounds: vertices each round added, rotating
  uint32_t pdone;                 // a pull round found that the round before it added nothing
  uint32_t err;                   // device-detected error code, 0 = none
  unsigned long long edges;       // in-edges gathered (statistic)
  unsigned long long affected;    // vertices marked before the first iteration
  uint32_t nfcnt;                 // DF / DF-P: vertices whose change exceeded D this iteration
  uint32_t xbcnt;                 // high out-degree vertices queued for block-wide expansion
  // FP32 refinement
  int k32;                        // FP32 sweeps in the current round (parity of e / ce)
  int inner_done;                 // the current round's FP32 sweeps have converged / hit the cap
  int rounds;                     // FP64 residual sweeps run
  unsigned int el32_bits[2];      // L-inf change of the FP32 sweep with parity k32 & 1 (bits of a float >= 0)
  unsigned int e32max_bits[2];    // L-inf of the correction it produced (personalized PageRank)
  int graph_rounds;               // bodies run by the CUDA-graph loop (its own bound)
  int graph_inner;                // bodies of a nested graph loop in the current outer body
  unsigned int el32_prev[2];      // FP32 rounds: the changes of the round's two previous sweeps (bits, 0: none)
  uint32_t q_head;                // DT closure queue (fr[0], length fcnt[0]): items claimed
  uint32_t q_done;                // ... and items whose out-neighbours are marked
};

// Device error codes (State::err bits).
constexpr uint32_t kErrClosureWait = 1u << 4;  // the DT closure's bounded wait ran out

// Internal mode of the update kernels: the FP64 residual sweep of the FP32
// refinement (reads the base ranks r[0] / c[0], writes the next iterate to
// r[1] and the residual, as FP32, to rho and e[0] / ce[0]).
constexpr int MODE_REFINE64 = 10;
// Flag added to DT / DF / DF-P: the same iterations on FP32 ranks and
// contributions (the refinement workspace's e[] and ce[]), the first phase of
// those modes under PRX_FP32_REFINE.
constexpr int MODE_F32 = 0x20;

// In-edges of the LOW class regrouped by source chunk: chunk k holds, for
// every vertex v, the in-edges whose source lies in [k*width, (k+1)*width),
// in the row's (ascending) order.  Offsets are chunk-major: the segment
// (k, v) is edg[off[k*(n+1) + v] .. off[k*(n+1) + v + 1]).  A sweep gathers
// one chunk at a time, so the contributions it reads fit in L2; the row's
// sum is carried across chunks in source order -- the reference's order.
struct ChunkLayout {
  uint32_t width = 0;             // vertices per source chunk, 0 = slot unused
  int K = 0;                      // number of chunks
  // Edge ids of hot sources (see GraphDev::hot_idx) are stored as
  // kHotFlag | (their index in the hot list): the sweep gathers those from
  // the dense hot copy of the contributions instead of c[].
  bool hot = false;
  uint64_t stamp = 0;             // last use (the least recently used slot is rebuilt)
  uint32_t* off = nullptr;        // K x (n + 1) offsets into edg
  uint32_t* edg = nullptr;
  // graphs with row segments: one layout per segment (rows [k * 2^S, ...),
  // K x (rows + 1) offsets each, relative to the segment's own edg)
  std::vector<uint32_t*> seg_off, seg_edg;
};

struct GraphDev {
  int device = 0;                 // device holding the arrays
  uint32_t n = 0;
  uint64_t m = 0;
  uint64_t m_cap = 0;             // capacity of the edge arrays
  uint32_t* xoff = nullptr;       // out-CSR (nullable)
  uint32_t* xedg = nullptr;
  uint32_t* xtoff = nullptr;      // in-CSR
  uint32_t* xtedg = nullptr;
  // Row segments, for edge arrays of 2^32 entries or more: rows
  // [k * 2^seg_shift, (k+1) * 2^seg_shift) form segment k, whose offsets are
  // 32-bit and relative to the segment's first edge, at xbase[k] / xtbase[k]
  // in the edge array.  Offset entries: n + nseg, row v's begin at
  // v + (v >> seg_shift) (seg_index).  One segment (seg_shift 32, bases null)
  // is the plain CSR.
  uint32_t seg_shift = 32;
  uint32_t nseg = 1;
  unsigned long long* xbase = nullptr;
  unsigned long long* xtbase = nullptr;
  std::vector<uint64_t> xseg0, xtseg0;  // host: first edge of each segment in the compact order
  std::vector<uint64_t> xpos, xtpos;    // host: the same as positions in the device arrays
  uint32_t* xtdat = nullptr;      // out-degree
  uint32_t* cls_list = nullptr;   // n ids: LOW ids, then MID, then HIGH (each ascending)
  uint32_t cls_begin[NCLS + 1] = {0, 0, 0, 0};
  uint64_t cls_edges[NCLS] = {0, 0, 0};  // in-edges per class
  uint32_t mid_max = kDefaultMidMax;
  uint32_t tuned_w64 = 0;         // source-chunk widths picked by prx_autotune (0: library default)
  uint32_t tuned_w32 = 0;
  int tuned_fetch = 0;            // L2 fetch granularity picked by prx_autotune (0: none)
  int tuned_int_adds = 0;         // integer-pipe adds of the FP64 sweep picked by prx_autotune (-1 none,
                                  // 1 .. 4; 0: not tuned)
  uint32_t* low_bm = nullptr;     // bitmap of the LOW class
  double* rcp = nullptr;          // RN(1 / outdeg) per vertex, for div_count
  float* rcp32 = nullptr;         // the same in FP32 (personalized PageRank sweeps)
  ChunkLayout lay[3];             // cached chunk layouts (rebuilt after a batch)
  // Hot sources: the vertices of largest out-degree (at most hot_cap of
  // them, out-degree at least twice the average), numbered 0 .. hot_n-1 in
  // id order.  Their contributions are copied after every sweep into a dense
  // array of hot_n values that stays in L2; edges from them are gathered
  // there (their values are the same, so sums are unchanged).  hot_idx: a
  // bitmap of the hot sources (ceil(n / 32) words), then per word the count
  // of hot sources in the words before it, so v's number is that count plus
  // the set bits below v in its word -- 8 bytes per 32 vertices, small
  // enough to stay in L2 while a layout scatter looks up every edge's
  // source.  Built on first use per graph version.
  uint32_t* hot_idx = nullptr;
  uint32_t* hot_list = nullptr;
  uint32_t hot_n = 0;
  uint32_t hot_cap = 0;
  bool hot_built = false;
  // batched personalized PageRank picks of prx_autotune_ppr (0: defaults):
  // rows of in-degree above ppr_low_max are cut into ppr_seg-edge segments
  uint32_t ppr_low_max = 0;
  uint32_t ppr_seg = 0;
  // edge weights (prx_graph_set_weights; dropped when a batch changes the edges)
  double* px = nullptr;           // P_uv = w_uv / W_u in out-CSR (xedg) order
  double* pt = nullptr;           // the same in in-CSR (xtedg) order
  double* wsum = nullptr;         // W_u = sum of u's out-edge weights
  unsigned long long* wseg = nullptr;  // row segments: each out-CSR segment's compact start (weights, dL/dw)
  uint32_t* ocls_list = nullptr;  // ids by out-degree class (rows of the out-CSR)
  uint32_t ocls_begin[NCLS + 1] = {0, 0, 0, 0};
  uint64_t ocls_edges[NCLS] = {0, 0, 0};
};

// Frees the edge weights of g (after a batch, or with the graph).
void drop_weights(GraphDev& g);

// The default LOW layout of a new graph (chunk width `width`, hot sources
// encoded when `hot`), built while its in-edges are still uploading: rows
// [piece_rows[p], piece_rows[p+1]) become usable when piece_ready[p] has
// fired; each piece is counted, scanned (with the totals of the pieces
// before it carried in) and scattered on stream s as soon as it has landed.
// Leaves the layout in the graph's cache; nothing for graphs of several row
// segments, more than 8 chunks or no layout to build.  Synchronizes s.
cudaError_t build_default_layout_pipelined(GraphDev& g, uint32_t width, bool hot, int pieces,
                                           const uint32_t* piece_rows, const cudaEvent_t* piece_ready, int sms,
                                           cudaStream_t s);

constexpr uint32_t kPfTable = 1u << 16;  // out-degrees whose DF-P factor is tabulated
constexpr uint32_t kHotFlag = 0x80000000u;
// The hot sources of g for a cap of `cap` vertices (0: none); graphs of 2^31
// vertices or more get none (their ids use the flag bit).
cudaError_t ensure_hot(GraphDev& g, uint32_t cap, int sms, cudaStream_t s);
void free_hot(GraphDev& g);

// Chunk layout of `width` vertices per chunk (built on first use, cached in
// three slots, the least recently used one rebuilt); width >= n means no
// chunking (*out = nullptr: the in-CSR itself) unless `hot`: ids of hot
// sources encoded (ensure_hot first), which always gives a layout, of one
// chunk of the LOW rows' edges if need be.
cudaError_t ensure_chunks(GraphDev& g, uint32_t width, int sms, cudaStream_t s, const ChunkLayout** out,
                          bool hot = false);
void free_chunks(GraphDev& g);

// Pointers a solve kernel needs.  Passed by value.
struct SolveArgs {
  const uint32_t* xoff;
  const uint32_t* xedg;
  const uint32_t* xtoff;
  const uint32_t* xtedg;
  const unsigned long long* xbase;   // row segments (see GraphDev); null: one segment
  const unsigned long long* xtbase;
  uint32_t seg_shift;
  const uint32_t* xtdat;
  const uint32_t* cls_list;       // static classes (see GraphDev)
  double* r[2];                   // FP64 ranks, ping-pong by iteration parity
  double* c[2];                   // FP64 contributions r/outdeg, ping-pong
  double* ch[2];                  // dense copies of the hot sources' c[p] (GraphDev::hot_idx)
  const uint32_t* hot_list;
  uint32_t hot_n;
  uint32_t* bm[3];                // affected bitmaps: iteration k uses bm[k%3] (cur), bm[(k+1)%3] (next)
  uint32_t* naff;                 // bitmap of seeded sources (marking)
  uint32_t* list[2][NCLS];        // dynamic: affected MID / HIGH vertices queued per iteration (list[0])
  uint32_t* xl;                   // marking: queued sources
  uint32_t* xb;                   // high out-degree vertices to expand block-wide
  uint32_t* nf[2];                // DF / DF-P: bitmap of vertices whose change exceeded D, by parity
  uint32_t* fr[3];                // DT closure frontiers: level L reads fr[L % 3], fills fr[(L+1) % 3]
  float* rho;                     // FP32 refinement: residual of the base ranks
  float* e[2];                    // FP32 refinement: correction, ping-pong
  float* ce[2];                   // FP32 refinement: correction / outdeg, ping-pong
  const uint32_t* low_bm;         // LOW-class bitmap
  const double* rcp;              // RN(1 / outdeg)
  uint32_t* ever;                 // FP32 dynamic phase: vertices updated at least once
  double* pf;                     // DF-P: 1 / (1 - P/d) per vertex (launch_prune_factor)
  double* pf_tab;                 // the same per out-degree d < kPfTable, formed once per solve
  double* acc64;                  // partial row sums carried between chunk passes (FP64)
  float* acc32;                   // the same for the FP32 sweeps
  State* st;
  uint32_t n;
  uint32_t mid_max;
  uint32_t pull_threshold;        // expand by pulling when more than this many vertices changed by > D
  uint32_t int_adds;              // FP64 LOW sweeps: adds of every four run on the integer pipes (0..4)
  double C0, P, D, C;
};

// ---- launchers (prx_update.cu) ------------------------------------------
void launch_init_ranks(const SolveArgs& a, const double* q, bool dynamic, cudaStream_t s);
// FP32 dynamic phase: e[0] = e[1] = (float)q, ce = e / outdeg.
void launch_init_ranks32(const SolveArgs& a, const double* q, cudaStream_t s);
// DF-P: the per-vertex factor 1 / (1 - P/d) of the closed-form update, into pf.
void launch_prune_factor(const SolveArgs& a, cudaStream_t s);
// After it: r[0] = (double)e[parity] where `ever` is set (else q, already in
// r[0]), c[0] = r[0] / outdeg; then the control block is reopened for the
// FP64 refinement (done only if the iteration cap was reached).
void launch_commit_dyn32(const SolveArgs& a, int parity, cudaStream_t s);
// Rank update of one in-degree class; false if nothing was launched.  For
// LOW, `lay` (may be null: no chunking) selects the chunk layout and one
// launch per chunk is made.
bool launch_update_class(const SolveArgs& a, const GraphDev& g, int mode, int cls, const ChunkLayout* lay, int sms,
                         cudaStream_t s);
void launch_finalize(const SolveArgs& a, int mode, cudaStream_t s);
// ch[p] <- the hot sources' c[p] (parity < 0: the parity the running
// iteration wrote); false when the solve uses no hot copy.
bool launch_hot_copy(const SolveArgs& a, int parity, int sms, cudaStream_t s);
// Adds of every four in a full step of the FP64 LOW sweep that run on the
// integer pipes when prx_options.int_adds is 0 and the graph is not tuned:
// one.  Static measured 0.4-7% faster on the 50M web-like graph (whose sweep
// DRAM and L1 also hold back; two or more cost more there than they save)
// and 5% faster on the 4096^2 grid (three: 17%), DF and DF-P within 2%.
constexpr uint32_t kDefaultIntAdds = 1;
// Hot-source cap when prx_options.hot_sources is 0: 32 MB of FP64 values.
constexpr uint32_t kDefaultHotCap = 4u << 20;
// Source-chunk width of the FP64 sweeps when prx_options.chunk_vertices is 0
// and the graph is untuned: 200 MB of FP64 contributions per chunk.
constexpr uint32_t kDefaultChunk64 = (200u << 20) / sizeof(double);

// ---- FP32 refinement (prx_refine.cu) --------------------------------------
// FP64 residual sweep of one in-degree class (update kernels in MODE_REFINE64).
bool launch_refine_sweep64(const SolveArgs& a, const GraphDev& g, int cls, const ChunkLayout* lay, int sms,
                           cudaStream_t s);
void launch_refine_finalize64(const SolveArgs& a, cudaStream_t s);
// The refinement loop's conditional nodes: arm before a node, cond at the end
// of its body (inner: the FP32 round, outer: the FP64 residual sweeps, at
// most cap bodies).
void launch_refine_arm(cudaGraphConditionalHandle h, const SolveArgs& a, bool inner, cudaStream_t s);
void launch_refine_cond(cudaGraphConditionalHandle h, const SolveArgs& a, bool inner, int cap, cudaStream_t s);
// One FP32 correction sweep of one class, and its finalize.
bool launch_sweep32(const SolveArgs& a, const GraphDev& g, int cls, const ChunkLayout* lay, int sms, cudaStream_t s);
void launch_finalize32(const SolveArgs& a, cudaStream_t s);
// x_b += e; c_b = x_b / outdeg.
void launch_refine_commit(const SolveArgs& a, int sms, cudaStream_t s);
// Round 0 of FP32 sweeps on the initial ranks in r[0] (x_b = 0, rho = C0).
void launch_refine_round0(const SolveArgs& a, int sms, cudaStream_t s);

// DF / DF-P expansion after an iteration's updates: push from the changed
// vertices or pull into the unmarked ones, chosen on the device.
void launch_expand_iteration(const SolveArgs& a, int sms, cudaStream_t s);
// Block-per-vertex expansion of the queued high out-degree vertices into
// bitmap `target` (0..2), or into the next-iteration bitmap when target < 0.
void launch_expand_big(const SolveArgs& a, int target, int sms, cudaStream_t s);

// ---- launchers (prx_mark.cu) --------------------------------------------
void launch_mark_seed(const SolveArgs& a, const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                      const uint32_t* insu, uint64_t ni, int sms, cudaStream_t s);
void launch_expand_seeds(const SolveArgs& a, int sms, cudaStream_t s);
void launch_frontier_from_bitmap(const SolveArgs& a, int sms, cudaStream_t s);
// DT closure by a work queue (frontier 0 holds the DF marking, its slots
// past the count set to all ones): persistent warps take reached vertices
// and mark their out-neighbours, until nothing is left, or until the queue
// holds more than switch_at vertices and eight times those done (a closure
// exploding in few steps, left to pull rounds).
void launch_closure_queue(const SolveArgs& a, uint32_t switch_at, int sms, cudaStream_t s);
// One DT closure round by pulling: every vertex not yet reached that has a
// reached in-neighbour joins (no-op once a round added nothing).
void launch_closure_pull(const SolveArgs& a, uint32_t round, int sms, cudaStream_t s);
void launch_popcount(const uint32_t* bm, uint32_t n, unsigned long long* out, int sms, cudaStream_t s);
void launch_flags_from_bitmap(const uint32_t* bm, uint8_t* out, uint32_t n, cudaStream_t s);
void launch_state_reset(State* st, int max_iter, double tol, cudaStream_t s);

// ---- graph construction (prx_graph.cu) ----------------------------------
// Degree classes, LOW bitmap and reciprocals of g's current arrays; the
// cached layouts and hot sources are dropped unless keep_layouts (a batch
// apply that carried them to the new version).
cudaError_t build_classes(GraphDev& g, int sms, cudaStream_t s, bool keep_layouts = false);
// The LOW-class bitmap and the reciprocal out-degrees (FP64 and FP32) of a
// graph version, by kernels alone (build_classes runs them too).
void launch_vertex_tables(const uint32_t* xtoff, uint32_t shift, const uint32_t* xtdat, uint32_t n, uint32_t* low_bm,
                          double* rcp, float* rcp32, int sms, cudaStream_t s);
// A new graph takes the picks prx_autotune made earlier in this process for a
// graph of the same signature, if any (prx_tune.cu).
cudaError_t tune_apply_cached(GraphDev& g, int sms, cudaStream_t s);
// Ids of the rows of `off` by length class (LOW, MID, HIGH; each ascending)
// into list (n), their bounds and the edges of each class.
cudaError_t build_class_lists(const uint32_t* off, uint32_t shift, uint32_t n, uint32_t mid_max, uint32_t* list,
                              uint32_t begin[NCLS + 1], uint64_t edges[NCLS], int sms, cudaStream_t s);
// b: device array [du | dv | iu | iv | tdk | tdv | tik | tiv]; t* = batch sorted by (v, u)
cudaError_t apply_batch_device(GraphDev& g, const uint32_t* b, uint64_t nd, uint64_t ni, int sms, cudaStream_t s);
// The arrays of one graph version (a plain CSR pair and the out-degrees).
struct CsrSet {
  uint32_t *xoff, *xedg, *xtoff, *xtedg, *xtdat;
};

// The LOW layout of `rows` rows in K source chunks of `width` vertices into
// caller buffers: K x (rows + 1) offsets, edge ids (edge_slots of the LOW
// edges), scan workspace of scan_ws_words(K x (rows + 1)) words; edge ids of
// hot sources encoded when hot_idx (GraphDev::hot_idx of a graph of
// 32 x hot_words vertices at most) is not null.  Kernels only.
cudaError_t build_layout_into(const uint32_t* off, const uint32_t* edg, const uint32_t* low_bm, uint32_t rows,
                              uint32_t width, int K, const uint32_t* hot_idx, uint32_t hot_words, uint32_t* lay_off,
                              uint32_t* lay_edg, uint32_t* scan_ws, int sms, cudaStream_t s);

// Workspace of apply_batch_graph for n vertices and batches of at most bmax
// edges (deletions plus insertions), carved from words(n, bmax) words.
struct ApplyWs {
  int32_t* delta;
  uint32_t *touched, *ranges, *cnt, *trow, *big, *scan_off, *scan_cnt;
  unsigned long long* nbig;
  static size_t words(uint32_t n, uint32_t bmax);
  ApplyWs(uint32_t* base, uint32_t n, uint32_t bmax);
};

// Apply a tidy batch (b: [du | dv | iu | iv | tdk | tdv | tik | tiv] as for
// apply_batch_device) to the plain CSRs src, writing dst (edge arrays large
// enough for the new count): the kernels of apply_batch_device with every
// count kept on the device -- no allocation and no host synchronisation, so
// the sequence can be captured into a conditional node's body.  The batch
// must have been checked (launch_batch_check).
cudaError_t apply_batch_graph(const CsrSet& src, const CsrSet& dst, uint32_t n, const uint32_t* b, uint32_t nd,
                              uint32_t ni, const ApplyWs& w, int sms, cudaStream_t s);
// The cached LOW layout l of a plain graph's previous version carried to
// its new version (in-CSR xtoff / xtedg): untouched rows' segments copied as
// shifted runs, the touched rows (bitmap `touched`, ascending list trow of T
// rows, or *Tp when Tp is not null) scattered again; new_off: K x (n + 1),
// new_edg: room for the new LOW edges, scan_ws: scan_ws_words(K x (n + 1)).
// Kernels only.
cudaError_t carry_layout(const ChunkLayout& l, const uint32_t* xtoff, const uint32_t* xtedg, uint32_t n,
                         const uint32_t* touched, const uint32_t* trow, uint32_t T, const uint32_t* Tp,
                         const uint32_t* hot_idx, uint32_t* new_off, uint32_t* new_edg, uint32_t* scan_ws, int sms,
                         cudaStream_t s);

// Sets bits of *err when batch b ([du | dv | iu | iv]) is not a tidy batch
// for the plain CSR xoff / xedg of n vertices: 8 an id >= n, 4 a list not
// strictly ascending in (u, v), then (only if neither) 1 a deletion is
// missing, 2 an insertion exists.  A set *err on entry skips the row reads.
void launch_batch_check(const uint32_t* xoff, const uint32_t* xedg, uint32_t n, const uint32_t* b, uint32_t nd,
                        uint32_t ni, uint32_t* err, int sms, cudaStream_t s);

cudaError_t exclusive_scan_u32(uint32_t* data, uint32_t len, cudaStream_t s);
// The same with a caller's workspace of scan_ws_words(len) words: no
// allocation, so it can be captured into a conditional node's body.
uint32_t scan_ws_words(uint32_t len);
cudaError_t exclusive_scan_u32_ws(uint32_t* data, uint32_t len, uint32_t* sums, cudaStream_t s);

// Stable LSD radix sort of keys[0 .. count) on their bits [lo, hi), 8 at a
// time, ping-ponging with tmp (both with 2 keys of slack past count: the
// last tile's bulk copy is rounded up to 16 bytes); *out is the buffer that
// holds the result.  hist: radix_hist_words(count) words.  (prx_tidy.cu)
size_t radix_hist_words(uint32_t count);
cudaError_t radix_sort_u64(unsigned long long* keys, unsigned long long* tmp, uint32_t count, int lo, int hi,
                           uint32_t* hist, int sms, cudaStream_t s, unsigned long long** out);
// The batch lists ordered by (v, u) for the in-CSR: a stable sort by v of
// the (u, v)-sorted lists u / v into tk (= v) / tv (= u).  (prx_batch.cu)
cudaError_t batch_by_target(const uint32_t* u, const uint32_t* v, uint32_t count, uint32_t n, uint32_t* tk,
                            uint32_t* tv, int sms, cudaStream_t s);

// Graph arrays come from a stream-ordered pool of this library that keeps
// freed memory (release threshold: unlimited), so a graph built after another
// one was destroyed reuses its pages instead of mapping new ones.  Allocated
// on stream s and usable there at once; returned by cudaFreeAsync on a
// stream or by graph_free.
cudaError_t graph_alloc(void** p, size_t bytes, cudaStream_t s);
template <class T>
cudaError_t graph_alloc(T** p, size_t bytes, cudaStream_t s) {
  return graph_alloc(reinterpret_cast<void**>(p), bytes, s);
}
// Returns pool blocks (NULLs skipped) once all work queued on the device has
// finished, like cudaFree; cudaFree itself would leave the pool counting the
// blocks as in use.
void graph_free(std::initializer_list<void*> ps);
// Give the pool's free memory on device dev back to the driver.
cudaError_t graph_pool_trim(int dev);
// Bytes the pool holds from the driver and bytes handed out, now and at peak.
cudaError_t graph_pool_stats(int dev, uint64_t out[4]);
// Mismatches of div_count against the IEEE division (prx_selftest_division).
cudaError_t selftest_division(uint32_t dmax, uint32_t per, unsigned long long* bad_host, int sms, cudaStream_t s);

void set_error(const std::string& msg);

}  // namespace prx
