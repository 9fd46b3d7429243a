/*
 * pagerank_gb300.h -- C ABI of the GB300 PageRank library.
 *
 * Replaces the five solver templates of puzzlef/pagerank-cuda-dynamic
 * (inc/pagerankCuda.hxx) and the host-side marshalling they perform
 * (pagerankInvokeCuda, inc/pagerankCuda.hxx:713-849):
 *
 *   pagerankStaticCuda<PARTITION,FLAG>(x, xt, o)                 :864-875
 *   pagerankNaiveDynamicCuda<PARTITION,FLAG>(x, xt, q, o)        :891-901
 *   pagerankDynamicTraversalCuda<...>(x, xt, y, yt, del, ins, q, o)  :921-930
 *   pagerankDynamicFrontierCuda<...>(x, xt, y, yt, del, ins, q, o)   :950-959
 *   pagerankPruneDynamicFrontierCuda<...>(x, xt, y, yt, del, ins, q, o) :979-988
 *
 * all of which map onto prx_solve() with a prx_mode.  The C++ header
 * pagerankCudaGb300.hxx re-exposes those templates on top of this ABI.
 *
 * Graphs are dense CSR: vertex ids 0..n-1 in the reference's vertexKeys()
 * order (inc/properties.hxx:26-33), neighbours ascending per row (the order
 * LazyBitset keeps, inc/_bitset.hxx).  Offsets are 32-bit, so m < 2^32, the
 * same limit as the reference (O = uint32_t, inc/pagerankCuda.hxx:715).
 *
 * Every entry point returns a prx_status; none of them exits the process
 * (the reference's TRY_CUDA exits, inc/_cuda.hxx:136-150).  Host buffers
 * belong to the caller; device memory belongs to the context and the graph.
 * A context and the graphs made from it must be used from one host thread
 * at a time.
 */
#ifndef PAGERANK_GB300_H
#define PAGERANK_GB300_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PRX_OK = 0,
  PRX_EINVAL = 1,    /* bad argument or malformed graph / batch          */
  PRX_ENOMEM = 2,    /* device or host allocation failed                 */
  PRX_ECUDA = 3,     /* a CUDA call failed (see prx_last_error())         */
  PRX_ETIMEOUT = 4,  /* a bounded device-side wait gave up               */
  PRX_ERANGE = 5,    /* size beyond a documented limit                   */
  PRX_ESTATE = 6,    /* call not valid for this object (e.g. no out-CSR) */
  PRX_ENOCONV = 7    /* iteration cap reached before the L-inf test passed,
                        reported only with prx_options.require_convergence;
                        ranks and result are still written              */
} prx_status;

/* The reference's five solvers (inc/pagerankCuda.hxx:864-988). */
typedef enum {
  PRX_STATIC = 0,
  PRX_NAIVE_DYNAMIC = 1,
  PRX_DYNAMIC_TRAVERSAL = 2,
  PRX_DYNAMIC_FRONTIER = 3,
  PRX_PRUNE_DYNAMIC_FRONTIER = 4
} prx_mode;

typedef enum {
  PRX_FP64 = 0,         /* the drop-in: ranks and contributions in FP64, the
                           reference's summation order, bit-exact to the oracle */
  PRX_FP32_REFINE = 1   /* FP32 storage / gathers / accumulation of a correction,
                           FP64 base ranks, FP64 residual and convergence test.
                           DT / DF / DF-P first run their iterations on FP32
                           ranks, then FP64 sweeps over all vertices refine
                           that result until the L-inf test passes: the answer
                           is the converged ranks to the tolerance, not the
                           FP64 path's answer bit for bit */
} prx_precision;

typedef enum {
  PRX_LOOP_AUTO = 0,    /* CUDA graph with a device-side while loop if possible:
                           Static / ND / DT / DF / DF-P without per-launch
                           timing; otherwise the host-driven loop           */
  PRX_LOOP_HOST = 1,    /* host-driven loop, convergence read back in batches   */
  PRX_LOOP_GRAPH = 2    /* CUDA graph with a conditional while node             */
} prx_loop;

/* PagerankOptions<V> (inc/pagerank.hxx:24-55) plus the GB300 knobs. */
typedef struct {
  int    repeat;              /* times to repeat the timed solve [1]        */
  double tolerance;           /* L-inf convergence tolerance [1e-10]        */
  double frontier_tolerance;  /* DF / DF-P expansion tolerance [1e-6]       */
  double prune_tolerance;     /* DF-P pruning tolerance [1e-6]              */
  double damping;             /* damping factor [0.85]                      */
  int    max_iterations;      /* iteration cap [500]                        */
  int    precision;           /* prx_precision [PRX_FP64]                   */
  int    loop;                /* prx_loop [PRX_LOOP_AUTO]                   */
  int    partition;           /* the reference's PARTITION template flag;
                                 accepted for drop-in use, results are the
                                 same either way [0]                         */
  int    timing;              /* 1: time every rank-update launch with CUDA
                                 events (prx_result.update_*) [0]            */
  int    expansion;           /* DF / DF-P marking after each sweep: 0 picks
                                 push or pull per iteration, 1 always pushes
                                 from changed vertices, 2 always pulls into
                                 unmarked ones; the marked set is the same [0] */
  uint32_t chunk_vertices;    /* source-chunk width of the gathers of the
                                 in-degree <= 64 class: each sweep reads the
                                 contributions one chunk of this many source
                                 vertices at a time; 0 sizes chunks to 200 MB
                                 of FP64 / 48 MB of FP32 contributions, >= n
                                 disables chunking.  Results do not depend
                                 on it [0]                                  */
  int    refine_sweeps;       /* PRX_FP32_REFINE with DT / DF / DF-P, the
                                 FP32 phase: 0 runs full sweeps from q when
                                 the initial marking covers more than n/8
                                 vertices (the frontier bookkeeping would
                                 cost more than it skips), else the mode's
                                 own frontier iterations; 1 always full
                                 sweeps; 2 always the mode's iterations.
                                 Either way the FP64 refinement returns the
                                 ranks converged to the tolerance [0]       */
  int    l2_fetch_bytes;      /* L2 fetch granularity hint for the solve
                                 (cudaLimitMaxL2FetchGranularity, how many
                                 bytes a missed load brings into L2): 0 the
                                 autotuner's pick for the graph (none when
                                 untuned), 32 / 64 / 128 that many, -1 none.
                                 The process's setting is put back before
                                 the call returns; results do not depend on
                                 it [0]                                     */
  int    require_convergence; /* 1: a solve that stops at max_iterations
                                 with its last L-inf change not below the
                                 tolerance returns PRX_ENOCONV (after
                                 writing ranks and result); 0: PRX_OK, as
                                 the reference returns its ranks either
                                 way [0]                                    */
  int    hot_sources;         /* FP64 sweeps of every mode and of
                                 PRX_FP32_REFINE: the vertices of largest
                                 out-degree (at most this many, with
                                 out-degree at least twice the average) get
                                 their contributions copied after each sweep
                                 into a dense array that stays in L2, and
                                 the gathers of their out-edges read it: the
                                 same values, so results do not depend on
                                 it.  0: at most 4,194,304 (32 MB); -1: none;
                                 graphs of 2^31 vertices or more get none [0] */
  int    int_adds;            /* FP64 sweeps of the in-degree <= 64 class:
                                 how many of every four edge additions run
                                 on the integer pipes (a correctly rounded
                                 integer adder, the same bits as the FP64
                                 add) to unload GB300's FP64 pipe: 0 the
                                 autotuner's pick for the graph (one when
                                 untuned), -1 none, 1 .. 4.  Results do not
                                 depend on it [0]                           */
} prx_options;

/* PagerankResult<V> (inc/pagerank.hxx:64-113) minus the rank vector, which
 * goes to the caller's buffer.  Times are milliseconds averaged over repeat,
 * measured with CUDA events on the context's stream. */
typedef struct {
  int      iterations;
  float    time_ms;
  float    initialization_time_ms;
  float    marking_time_ms;
  float    computation_time_ms;
  uint64_t affected_initial;   /* vertices marked before the first iteration  */
  uint64_t edges_processed;    /* in-edges gathered over all iterations         */
  double   last_delta;         /* L-inf change of the last iteration            */
  int      refinements;        /* FP32_REFINE: outer FP64 residual checks run   */
  uint64_t kernel_launches;    /* kernels this library launched for the solve  */
  /* With prx_options.timing: per in-degree class (<= 64, warp, block) the
   * summed device time and count of rank-update launches (last repeat). */
  double   update_ms[3];
  uint32_t update_launches[3];
  /* the same for the FP32 correction sweeps of PRX_FP32_REFINE */
  double   update32_ms[3];
  uint32_t update32_launches[3];
} prx_result;

typedef struct prx_context prx_context;
typedef struct prx_graph prx_graph;

void        prx_options_default(prx_options* o);
const char* prx_status_string(int status);
/* Text of the last failure on this host thread ("" if none). */
const char* prx_last_error(void);

/* A context owns one CUDA stream on `device` and a workspace that grows on
 * demand.  cudaSetDeviceFlags(cudaDeviceMapHost) is not needed (the
 * reference sets it, inc/pagerankCuda.hxx:777). */
int prx_context_create(int device, prx_context** out);
int prx_context_destroy(prx_context* ctx);
/* The context's stream, as a cudaStream_t cast to void*. */
void* prx_context_stream(prx_context* ctx);

/* Every graph holds at most 2^32 - 2^24 vertices (PRX_ERANGE above). */

/* Upload a graph (the csrCreate*W / cudaMemcpy part of pagerankInvokeCuda,
 * inc/pagerankCuda.hxx:756-805).  xoff/xedg: out-CSR of the graph, needed by
 * the dynamic modes and prx_graph_apply_batch (may be NULL for Static / ND);
 * xtoff/xtedg: in-CSR (transpose); xtdat: out-degree of each vertex.  All
 * pointers are host pointers.  `validate` != 0 checks every offset and id. */
int prx_graph_create(prx_context* ctx, uint32_t n, uint64_t m,
                     const uint32_t* xoff, const uint32_t* xedg,
                     const uint32_t* xtoff, const uint32_t* xtedg,
                     const uint32_t* xtdat, int validate, prx_graph** out);
/* The same with 64-bit offsets, for graphs of 2^32 edges or more (288 GB of
 * HBM holds about 20 billion FP64 edges).  Rows are cut into segments of
 * 2^seg_shift rows whose edges are addressed with 32-bit offsets from the
 * segment's start; seg_shift 0 picks it (one segment, the plain CSR, while
 * m < 2^32), 1..32 forces it (PRX_ERANGE if a segment would hold 2^32 edges
 * or more).  Graphs with more than one segment support every solver mode,
 * the FP32 refinement, marking, autotuning and download (source chunks are
 * built per segment, for segments of 32 rows or more); batch apply, tidy and
 * generation, personalized PageRank and edge weights return PRX_ERANGE. */
int prx_graph_create64(prx_context* ctx, uint32_t n, uint64_t m,
                       const uint64_t* xoff, const uint32_t* xedg,
                       const uint64_t* xtoff, const uint32_t* xtedg,
                       const uint32_t* xtdat, int validate, uint32_t seg_shift, prx_graph** out);
int prx_graph_download64(prx_graph* g, uint64_t* xoff, uint32_t* xedg,
                         uint64_t* xtoff, uint32_t* xtedg, uint32_t* xtdat);
/* A graph may be destroyed before or after its context; every other call on
 * a graph needs its context alive.  Graph arrays come from a pool of this
 * library that keeps freed memory for the next graph on the device;
 * prx_release_cached_memory gives that memory back to the driver. */
int prx_graph_destroy(prx_graph* g);
int prx_release_cached_memory(int device);
/* That pool on `device`: bytes held from the driver and bytes in use, now and
 * at their peak (each output may be NULL; all 0 before the first graph). */
int prx_graph_pool_stats(int device, uint64_t* reserved, uint64_t* reserved_peak, uint64_t* used,
                         uint64_t* used_peak);
/* The L2 fetch granularity hint of this process's context on `device`
 * (cudaLimitMaxL2FetchGranularity: how many bytes a missed load brings into
 * L2).  *previous (may be NULL) receives the current value; bytes in 0..128
 * sets it, bytes < 0 only reads it.  A context limit, gone with the process. */
int prx_l2_fetch_granularity(int device, int bytes, int* previous);
/* Current vertex / edge counts (m changes with prx_graph_apply_batch). */
int prx_graph_size(const prx_graph* g, uint32_t* n, uint64_t* m);
/* Vertices and in-edges in each in-degree class of the rank update:
 * [0] in-degree <= 64 (thread per vertex), [1] up to the warp limit (warp per
 * vertex), [2] above it (block per vertex).  Either pointer may be NULL. */
int prx_graph_class_stats(const prx_graph* g, uint32_t vertices[3], uint64_t edges[3]);
/* Copy the graph back to host buffers (any pointer may be NULL). */
int prx_graph_download(prx_graph* g, uint32_t* xoff, uint32_t* xedg,
                       uint32_t* xtoff, uint32_t* xtedg, uint32_t* xtdat);

/* Apply a tidied batch on the device to both CSRs and the out-degrees:
 * deletions must exist, insertions must not, each list sorted by (u, v)
 * and free of duplicates -- the output of tidyBatchUpdateU
 * (inc/batch.hxx:200-208).  Same effect as applyBatchUpdateOmpU
 * (inc/batch.hxx:239-247) followed by transposeWithDegreeOmp
 * (inc/transpose.hxx:128-134).  Graphs with row segments
 * (prx_graph_create64) keep their segments, which move to new bases; each
 * must stay below 2^32 - 8 edges (PRX_ERANGE otherwise, graph unchanged).
 * Host pointers. */
int prx_graph_apply_batch(prx_graph* g,
                          const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                          const uint32_t* insu, const uint32_t* insv, uint64_t ni);

/* Solve with the ranks and batch in HOST memory.  The graph must already hold
 * the updated graph y / yt (as the reference's callers pass it).  q: previous
 * ranks (n doubles) or NULL for 1/n; Static ignores q.  deletions/insertions:
 * the tidied batch that produced the graph (dynamic modes; insv may be NULL).
 * ranks_out: n doubles.  res may be NULL. */
int prx_solve(prx_context* ctx, prx_graph* g, int mode,
              const uint32_t* delu, const uint32_t* delv, uint64_t nd,
              const uint32_t* insu, const uint32_t* insv, uint64_t ni,
              const double* q, const prx_options* o,
              double* ranks_out, prx_result* res);

/* Same, with q, ranks_out and the batch arrays in DEVICE memory (inputs
 * already resident in HBM).  Runs on the context's stream and returns after
 * the solve completed. */
int prx_solve_device(prx_context* ctx, prx_graph* g, int mode,
                     const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                     const uint32_t* insu, const uint32_t* insv, uint64_t ni,
                     const double* q, const prx_options* o,
                     double* ranks_out, prx_result* res);

/* K consecutive batch updates as ONE CUDA graph launch: for k = 0 .. K-1,
 * apply batch k to g (as prx_graph_apply_batch does) and solve `mode`
 * (PRX_DYNAMIC_FRONTIER or PRX_PRUNE_DYNAMIC_FRONTIER, FP64) from the
 * previous step's ranks (q for step 0) -- the reference driver's loop over
 * its batches (main.cu:88-147) without a host round trip between them.
 * Batch k deletes del_u/del_v[del_off[k] .. del_off[k+1]) and inserts
 * ins_u/ins_v[ins_off[k] .. ins_off[k+1]), each list sorted by (u, v) and
 * tidy against the graph as the batches before it left it.  del_off and
 * ins_off (K + 1 entries each) are HOST memory; the id arrays, q and
 * ranks_out (n doubles: the ranks after the last step) and ranks_each
 * (K x n doubles, row k after step k; may be NULL) are DEVICE memory.
 * res (K entries, may be NULL): per step its iterations, marking size,
 * edges, last change, launches, and its times from the device clock
 * (initialization: the check, the apply and the step's layout and ranks;
 * then marking; then computation: the iterations).  Plain
 * graphs (prx_graph_create) only; the steps gather through a source-chunk
 * layout rebuilt by kernels for every step and the hot sources of the graph
 * before the batches.  A batch that is not tidy ends
 * the sequence: PRX_EINVAL, *applied = the steps completed, and the graph
 * and ranks_out as the last of them left them. */
int prx_solve_batches_device(prx_context* ctx, prx_graph* g, int mode, uint32_t K,
                             const uint64_t* del_off, const uint32_t* del_u, const uint32_t* del_v,
                             const uint64_t* ins_off, const uint32_t* ins_u, const uint32_t* ins_v,
                             const double* q, const prx_options* o, double* ranks_out,
                             double* ranks_each, prx_result* res, uint32_t* applied);

/* tidyBatchUpdateU (inc/batch.hxx:152-208), on the device: against graph g
 * (created with its out-CSR, before the batch is applied), keep the
 * deletions that exist and the insertions that do not, sort each list by
 * (u, v) and drop duplicates.  Host arrays in and out; the outputs need room
 * for nd / ni edges, and *out_nd / *out_ni receive the tidied lengths.  The
 * result is what prx_graph_apply_batch takes. */
int prx_graph_tidy_batch(prx_context* ctx, prx_graph* g,
                         const uint32_t* del_u, const uint32_t* del_v, uint64_t nd,
                         const uint32_t* ins_u, const uint32_t* ins_v, uint64_t ni,
                         uint32_t* out_del_u, uint32_t* out_del_v, uint64_t* out_nd,
                         uint32_t* out_ins_u, uint32_t* out_ins_v, uint64_t* out_ni);

/* A random batch drawn and tidied on the device: nd_req deletions of
 * uniformly chosen existing non-self-loop edges and ni_req insertions of
 * uniform pairs, then tidied as prx_graph_tidy_batch does.  The same draws
 * (counter-based hashes of seed and index) and so the same batch as the host
 * generator prx_gen_batch on the graph's out-CSR.  Host output arrays with
 * room for nd_req / ni_req edges. */
int prx_graph_gen_batch(prx_context* ctx, prx_graph* g, uint64_t nd_req, uint64_t ni_req, uint64_t seed,
                        uint32_t* del_u, uint32_t* del_v, uint64_t* nd,
                        uint32_t* ins_u, uint32_t* ins_v, uint64_t* ni);

/* Build a graph on the device from an edge list (0-based ids < n, any order,
 * duplicates allowed): the out-CSR (rows ascending, duplicates merged), the
 * in-CSR and the out-degrees -- what the reference assembles on the host
 * with readTemporalOmpW (inc/snap.hxx:158-166, main.cu:167),
 * addSelfLoopsOmp (inc/selfLoop.hxx:60-66, main.cu:169; here when
 * self_loops != 0, a loop on every vertex) and transposeWithDegreeOmp
 * (inc/transpose.hxx:110-134, main.cu:170).  u, v: host arrays of `count`
 * ids.  Equivalent to prx_graph_create with those CSRs. */
int prx_graph_create_from_edges(prx_context* ctx, uint32_t n, const uint32_t* u, const uint32_t* v,
                                uint64_t count, int self_loops, prx_graph** out);
/* Same, with u and v in DEVICE memory (left unchanged). */
int prx_graph_create_from_edges_device(prx_context* ctx, uint32_t n, const uint32_t* u, const uint32_t* v,
                                       uint64_t count, int self_loops, prx_graph** out);

/* Run only the initial affected-vertex marking of a dynamic mode
 * (pagerankAffectedFrontierCuW :405-412 for DF / DF-P,
 * pagerankAffectedTraversalCuW :438-456 for DT) and copy the flags (n bytes,
 * 0/1) to host memory. */
int prx_mark_affected(prx_context* ctx, prx_graph* g, int mode,
                      const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                      const uint32_t* insu, uint64_t ni, uint8_t* flags_out);

/* ---- batched personalized PageRank (no counterpart in the reference) ---- */

/* Statistics of one batched personalized PageRank solve. */
typedef struct {
  int      iterations;        /* sweeps of the slowest column block        */
  int      fp64_sweeps;       /* FP64 sweeps, summed over column blocks     */
  int      fp32_sweeps;       /* FP32 correction sweeps (FP32_REFINE)       */
  int      refinements;       /* FP64 residual sweeps (FP32_REFINE)         */
  float    time_ms;           /* device time of the solve (CUDA events)     */
  double   last_delta;        /* largest final L-inf change of a block      */
  uint64_t kernel_launches;   /* kernels run, inside the graphs included    */
  uint64_t graph_launches;    /* CUDA graph launches: one per column block
                                 with the default loop, 0 with PRX_LOOP_HOST */
  uint32_t low_max;           /* rows of in-degree above this were cut ...  */
  uint32_t seg_edges;         /* ... into segments of this many in-edges
                                 (64 / 512, or prx_autotune_ppr's picks)    */
} prx_ppr_result;

/* Personalized PageRank of nvec teleport vectors on graph g.  Vector k
 * teleports uniformly to the seeds seeds[seed_off[k] .. seed_off[k+1])
 * (host arrays; non-empty sets of ids < n, a repeated id counts twice):
 *   r_k = (1 - damping) t_k + damping * A^T D^-1 r_k,
 * iterated by Jacobi sweeps from r_k = t_k until the largest change of one
 * sweep over the vertices and the vectors of a block of 64 vectors is below
 * o->tolerance, or o->max_iterations sweeps.  o->precision PRX_FP64 stores
 * and sums in FP64; PRX_FP32_REFINE runs the correction sweeps in FP32 with
 * FP64 residuals (the FP64 residual decides convergence).  Vectors are
 * solved 64 at a time; each block's iteration loop is one CUDA graph launch
 * (a conditional WHILE node, and for the refinement a nested one over each
 * round's FP32 sweeps), or with o->loop = PRX_LOOP_HOST a host loop over the
 * same kernels (the same results).  ranks_out: n * nvec doubles in host
 * memory, vertex-major (ranks_out[v * nvec + k]).  Other options are
 * ignored. */
int prx_solve_ppr_batched(prx_context* ctx, prx_graph* g, uint32_t nvec,
                          const uint32_t* seed_off, const uint32_t* seeds,
                          const prx_options* o, double* ranks_out, prx_ppr_result* res);

/* Picks of prx_autotune_ppr (no counterpart in the reference). */
typedef struct {
  uint32_t low_max;           /* rows up to this in-degree: one warp per vertex */
  uint32_t seg_edges;         /* longer rows: segments of this many in-edges     */
  float    ms_per_solve;      /* the winner's time for the trial solve           */
  int      trials;            /* candidate pairs timed                           */
} prx_ppr_tune_result;

/* Times short FP32-refined batched solves on g (64 vectors; 1 FP64 and 5
 * FP32 sweeps, best of two) over the warp-per-vertex bound (64, 256, 1024)
 * and the segment width of longer rows (256, 512, 1024, 2048 in-edges), and
 * keeps the fastest pair on g: later prx_solve_ppr_batched calls on g use it
 * (results change only by rounding: the sums' grouping follows the split).
 * Not for graphs with row segments (PRX_ERANGE). */
int prx_autotune_ppr(prx_context* ctx, prx_graph* g, prx_ppr_tune_result* out);

/* The same with ranks_out in device memory (seeds stay host arrays). */
int prx_solve_ppr_batched_device(prx_context* ctx, prx_graph* g, uint32_t nvec,
                                 const uint32_t* seed_off, const uint32_t* seeds,
                                 const prx_options* o, double* ranks_out, prx_ppr_result* res);

/* ---- weighted PageRank and its adjoint (no counterpart in the reference) --
 * Edge u -> v carries a weight w_uv > 0, rows are normalised
 * (P_uv = w_uv / W_u, W_u = sum_v w_uv) and
 *   r = (1 - damping) t + damping P^T r.
 * The adjoint of a loss L(r) with g = dL/dr solves
 *   lambda = damping P lambda + g
 * by the same pull kernels on the out-CSR (the reversed graph) and gives
 *   dL/dw_uv = (r_u / W_u)(damping lambda_v - lambda_u + g_u),
 *   dL/dt = (1 - damping) lambda,  dL/ddamping = lambda . (P^T r - t).
 * Both solves are Jacobi iterations stopped by the reference's L-inf test
 * (o->tolerance, o->max_iterations); they run in FP64.  Pointers are device
 * pointers unless stated; the calls return after their work finished. */

/* Attach weights w (m floats, device, in out-CSR order: the weight of edge
 * xedg[j] at w[j]) to a graph created with its out-CSR.  A batch applied to
 * the graph drops the weights. */
int prx_graph_set_weights(prx_context* ctx, prx_graph* g, const float* w);

/* Weighted PageRank: t (n, NULL = uniform 1/n) is the teleport vector, r0
 * (n, NULL = t) the starting ranks; the converged ranks go to r (n).
 * res->iterations, last_delta, time_ms and kernel_launches are set. */
int prx_solve_weighted(prx_context* ctx, prx_graph* g, const double* t, const double* r0,
                       const prx_options* o, double* r, prx_result* res);

/* Adjoint of the weighted solve at converged ranks r (n) for teleport t (n,
 * NULL = uniform) and loss gradient gl = dL/dr (n).  Outputs, each
 * optional: lambda (n), grad_w (m, out-CSR order), grad_t (n) and
 * grad_alpha (one double in HOST memory).  res->iterations counts the
 * adjoint sweeps. */
int prx_adjoint(prx_context* ctx, prx_graph* g, const double* t, const double* r, const double* gl,
                const prx_options* o, double* lambda, double* grad_w, double* grad_t, double* grad_alpha,
                prx_result* res);

/* ---- autotuning (no counterpart in the reference) ---------------------- */

typedef struct {
  uint32_t mid_max;           /* in-degree above which a vertex gets a block, not a warp */
  uint32_t chunk_vertices64;  /* source-chunk width of the FP64 sweeps (>= n: none)    */
  uint32_t chunk_vertices32;  /* the same for the FP32 sweeps of PRX_FP32_REFINE        */
  float    ms_per_iteration64;
  float    ms_per_iteration32;
  int      trials;            /* trial solves run (0 when taken from the cache)         */
  int      cached;            /* 1: picks reused for a graph of the same signature      */
  int      l2_fetch_bytes;    /* L2 fetch granularity of the solves (32, 64 or 128)     */
  int      int_adds;          /* integer-pipe adds of every four in the FP64 sweeps
                                 (-1 none, 1 .. 4; 0 from a cache line without it)   */
} prx_tune_result;

/* Times short Static solves on g (FP64 and FP32 refinement, 3 iterations
 * each, best of two) over the MID / HIGH in-degree boundary (1024, 4096,
 * 16384), the source-chunk widths (none, 200/128/64 MB of FP64
 * contributions, 96/48/24 MB of FP32 ones) and the L2 fetch granularity (32,
 * 64, 128 bytes; FP64 plus FP32 time), then prx_options.int_adds (none,
 * 1 .. 4; FP64 time), and keeps the fastest on g: later solves with
 * chunk_vertices = 0, l2_fetch_bytes = 0 and int_adds = 0 use them.  Results
 * do not depend on these parameters.  Picks are cached per graph signature (n, m, in-degree class
 * sizes) in the process and, when cache_path is not NULL, in that text file
 * (read before, rewritten after).  A graph created later in the process with
 * the same signature takes the cached picks when it is built. */
int prx_autotune(prx_context* ctx, prx_graph* g, const char* cache_path, prx_tune_result* out);

/* Diagnostic with no counterpart in the reference: counts, on the context's
 * device, the dividends a and out-degrees d (d = 1 .. dmax, `per` values of a
 * per d, spread over 2^-40 .. 2^2) for which the library's three-operation
 * division by a precomputed reciprocal differs from the IEEE division a / d.
 * The solvers divide ranks by out-degrees that way.  Each sample also checks
 * the multiply-first comparisons of a relative change with a tolerance
 * (DF / DF-P) against the comparison of the correctly rounded quotient, in
 * the band where the two are closest. */
int prx_selftest_division(prx_context* ctx, uint32_t dmax, uint32_t per, unsigned long long* mismatches);

/* Static FP64 PageRank that allocates no memory.  No counterpart in the
 * reference: it serves callers that may not allocate device memory behind
 * their own allocator (a serving process that reserves its HBM up front, a
 * plugin host that owns all device memory).  The caller passes the in-CSR,
 * the out-degrees and the ranks buffer (n doubles), all in device memory;
 * stream is a cudaStream_t or NULL.  Results and iteration count equal
 * prx_solve(PRX_STATIC) bit for bit.  Scratch is one static device array
 * sized for PRX_NOALLOC_MAX_VERTICES vertices (24 MiB per GPU that uses the
 * call, held until the process exits); larger n returns PRX_ERANGE.  All
 * calls share that array, so calls that overlap on the GPU race and must be
 * ordered by the caller.  Every call looks the array's device address up
 * in the calling thread's current context (no allocation); the first call in
 * a context is where the CUDA loader places the array, so make it before any
 * stream capture.  Preconditions, as prx_graph_create checks them for the
 * regular path: xtoff[0] = 0, xtoff non-decreasing, xtoff[n] = m, every
 * xtedg id < n, every xtdat >= 1 (each vertex's out-degree, its self-loop
 * included).  A first or last offset that breaks them is caught on the
 * device before any sweep and returns PRX_EINVAL; the rest is the caller's
 * promise (a bad id reads out of bounds).  Returns after the solve
 * finished. */
#define PRX_NOALLOC_MAX_VERTICES 1048576u
int prx_static_solve_noalloc(uint32_t n, uint64_t m,
                             const uint32_t* xtoff, const uint32_t* xtedg, const uint32_t* xtdat,
                             double damping, double tolerance, int max_iterations,
                             double* ranks, int* iterations, void* stream);

/* ---- host-side graph utilities (C++ / OpenMP; no device work) ---------- */

/* A CSR allocated by the library; free with prx_host_csr_free. */
typedef struct {
  uint32_t  n;
  uint64_t  m;
  uint32_t* off;   /* n+1 */
  uint32_t* edg;   /* m   */
} prx_host_csr;

void prx_host_csr_free(prx_host_csr* g);

/* R-MAT (a, b, c; d = 1-a-b-c) with n = 2^scale and edge_factor*n draws,
 * duplicates removed, a self-loop on every vertex, rows ascending. */
int prx_gen_rmat(int scale, int edge_factor, double a, double b, double c,
                 uint64_t seed, prx_host_csr* out);
/* Web-like graph: out-degree floor(dmin * U^(-1/(alpha-1))) capped at dmax,
 * a fraction `local` of each row's targets within +/-window of the source,
 * the rest uniform; duplicates removed; self-loops on all vertices. */
int prx_gen_weblike(uint32_t n, double alpha, double dmin, uint32_t dmax,
                    double local, uint32_t window, uint64_t seed, prx_host_csr* out);
/* w x w grid, 4-neighbour edges both ways, a diagonal edge pair (both ways)
 * from a fraction `diag` of the vertices, self-loops on all vertices. */
int prx_gen_grid(uint32_t w, double diag, uint64_t seed, prx_host_csr* out);
/* Random batch on x: ni_req insertions of uniform pairs and nd_req deletions
 * of uniformly chosen existing non-self-loop edges, then tidied (filtered by
 * existence, sorted, unique; inc/batch.hxx:152-208).  Arrays are allocated
 * by the library; free with prx_host_free. */
int prx_gen_batch(const prx_host_csr* x, uint64_t nd_req, uint64_t ni_req, uint64_t seed,
                  uint32_t** delu, uint32_t** delv, uint64_t* nd,
                  uint32_t** insu, uint32_t** insv, uint64_t* ni);
/* tidyBatchUpdateU on caller arrays, in place; returns new lengths. */
int prx_host_tidy_batch(const prx_host_csr* x, uint32_t* delu, uint32_t* delv, uint64_t* nd,
                        uint32_t* insu, uint32_t* insv, uint64_t* ni);
/* Out-CSR of x with a tidied batch applied (host). */
int prx_host_apply_batch(const prx_host_csr* x,
                         const uint32_t* delu, const uint32_t* delv, uint64_t nd,
                         const uint32_t* insu, const uint32_t* insv, uint64_t ni,
                         prx_host_csr* y);
/* Edge-list readers.  Ids in the files are 1-based; the arrays returned are
 * 0-based, allocated by the library (free with prx_host_free).
 *
 * SNAP temporal text ("u v [t]" per line), read in consecutive pieces as the
 * reference's driver does (main.cu:167 reads the first 90% of the lines,
 * main.cu:83 each batch): prx_edge_reader_next reads the next `size` lines
 * (fewer at the end of the file); a line that does not start with two
 * unsigned integers ends the piece, as in readTemporalDo
 * (inc/snap.hxx:41-52).  Ids must lie in 1..rows (PRX_EINVAL otherwise);
 * symmetric != 0 adds (v, u) after each (u, v). */
typedef struct prx_edge_reader prx_edge_reader;
int prx_edge_reader_open(const char* path, prx_edge_reader** out);
int prx_edge_reader_next(prx_edge_reader* r, uint32_t rows, uint64_t size, int symmetric,
                         uint32_t** u, uint32_t** v, uint64_t* count, uint64_t* lines);
int prx_edge_reader_close(prx_edge_reader* r);
/* MatrixMarket coordinate file (readMtxDo, inc/mtx.hxx:119-135; header by
 * readMtxHeader, inc/mtx.hxx:39-54): n = max(rows, cols); a symmetric or
 * skew-symmetric matrix gives both (u, v) and (v, u); a file that is not
 * "matrix coordinate" gives n = 0 and no edges; reading stops at the first
 * line without two unsigned integers.  Ids must lie in 1..n. */
int prx_read_mtx(const char* path, uint32_t* n, uint32_t** u, uint32_t** v, uint64_t* count);
/* The edges as text, "u v\n" per edge with 1-based ids (what the readers
 * take); *text is allocated by the library, free with prx_host_free. */
int prx_format_edges(const uint32_t* u, const uint32_t* v, uint64_t count, char** text, uint64_t* bytes);

/* Edge-list text parsed on the DEVICE and built into a graph there (the
 * same lines and the same edges as the host readers above, then what
 * prx_graph_create_from_edges does with them).  Symmetric != 0 adds (v, u)
 * after each (u, v); self_loops != 0 adds a loop on every vertex.
 *
 * prx_graph_create_from_text: up to `size` lines of text[0 .. bytes), host
 * memory, ids in 1..rows, the last line may lack its newline; *lines and
 * *used receive the lines and bytes consumed (either may be NULL).
 * prx_edge_reader_next_graph: the next `size` lines of an open reader, as
 * prx_edge_reader_next reads them (the reference's first 90% read,
 * main.cu:167, builds its graph this way).
 * prx_graph_create_from_mtx: a whole MatrixMarket coordinate file, n =
 * max(rows, cols) (*n_out may be NULL). */
int prx_graph_create_from_text(prx_context* ctx, const char* text, uint64_t bytes, uint32_t rows, uint64_t size,
                               int symmetric, int self_loops, prx_graph** out, uint64_t* lines, uint64_t* used);
int prx_edge_reader_next_graph(prx_edge_reader* r, prx_context* ctx, uint32_t rows, uint64_t size, int symmetric,
                               int self_loops, prx_graph** out, uint64_t* lines);
int prx_graph_create_from_mtx(prx_context* ctx, const char* path, int self_loops, prx_graph** out,
                              uint32_t* n_out);
/* One result line in the reference driver's log format (main.cu:54-61):
 * "{-<del>/+<ins> batchf, <batch> batchi, <threads> threads} -> {<time>ms,
 * <init>ms init, <mark>ms mark, <comp>ms comp, <iter> iter, <err> err}
 * <technique>", without a newline.  Returns what snprintf returns (the
 * length the full line needs), or -PRX_EINVAL. */
int prx_format_glog(char* buf, size_t len, double deletions_fraction, double insertions_fraction,
                    int batch_index, int threads, const prx_result* r, double err, const char* technique);
/* In-CSR (sources ascending) and out-degrees of x; xtdat has n entries. */
int prx_host_transpose(const prx_host_csr* x, prx_host_csr* xt, uint32_t* xtdat);
void prx_host_free(void* p);

#ifdef __cplusplus
}
#endif
#endif
