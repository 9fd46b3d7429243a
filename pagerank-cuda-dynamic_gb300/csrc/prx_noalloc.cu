// prx_noalloc.cu -- Static FP64 PageRank that allocates no device memory.
//
// Who needs this: a caller whose process hands out device memory only through
// its own allocator or a fixed budget -- a serving process that reserves its
// HBM up front, or a host application embedding this library as a plugin --
// cannot let a library call cudaMalloc / cudaFree behind its back (those
// calls also synchronize the device, which such callers avoid).  The caller
// owns the graph arrays and the output ranks; everything else the solve needs
// lives in one file-scope device array that the CUDA loader reserves once per
// GPU when this module is first used, and keeps until the process exits.
//
// Limits and sharing:
//  - at most PRX_NOALLOC_MAX_VERTICES vertices (the array holds a second rank
//    buffer and two contribution buffers of that length, 24 MiB in all);
//  - every call, on every stream, uses the same array: two calls that can
//    overlap on one GPU race with each other and corrupt both results; order
//    them on one stream or with events;
//  - the array keeps whatever the last call left; each call re-initialises
//    everything it reads (control block, ranks, contributions) before use.
//  - Every call looks the array's device address up (cudaGetSymbolAddress,
//    which allocates nothing) in the context current on the calling thread,
//    so a device reset or another context on the same device never leaves a
//    stale address behind.  The first call in a context is also where the
//    CUDA loader places the array, so make it before any stream capture.
//
// Preconditions (as prx_graph_create checks them for the regular path):
// xtoff[0] = 0, xtoff non-decreasing, xtoff[n] = m, every xtedg id below n,
// every xtdat (out-degree, self-loop included) at least 1.  The first and
// last offsets are checked on the device before any sweep (PRX_EINVAL); the
// rest is the caller's promise.
//
// Results are bit-identical to prx_solve(PRX_STATIC): the same sums in the
// same order (front to back for in-degree <= 64, 256 strided partial sums
// and a halving tree above that, inc/pagerankCuda.hxx:87-109, 162-188 and
// inc/_cuda.hxx:541-551), the same fma epilogue and stopping rule.
#include <string>
#include "prx_device.cuh"

namespace {

constexpr int kHeadDoubles = 32;  // 256-byte control block before the vectors
constexpr size_t kScratchDoubles = kHeadDoubles + 3 * (size_t)PRX_NOALLOC_MAX_VERTICES;

// The device scratch.  In host code this name is only a stand-in for the
// symbol; kernels get the address cudaGetSymbolAddress returned.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct NaState {
  unsigned long long el_bits[2];
  int iter;
  int done;
  int max_iter;
  int bad;      // the offsets failed the first / last check
  double tol;
};
static_assert(sizeof(NaState) <= kHeadDoubles * sizeof(double), "control block too large");

struct NaArgs {
  const uint32_t* xtoff;
  const uint32_t* xtedg;
  const uint32_t* xtdat;
  double* out;       // caller's ranks: rank buffer of parity 0
  double* scratch;   // device address of g_noalloc_scratch
  uint32_t n;
  double C0, P;
  __device__ NaState* st() const { return reinterpret_cast<NaState*>(scratch); }
  __device__ double* rank(int p) const { return p ? scratch + kHeadDoubles : out; }
  __device__ double* contrib(int p) const {
    return scratch + kHeadDoubles + (size_t)PRX_NOALLOC_MAX_VERTICES * (1 + p);
  }
};

__global__ void k_na_reset(NaArgs a, uint32_t m, int max_iter, double tol) {
  NaState* s = a.st();
  s->el_bits[0] = s->el_bits[1] = 0;
  s->iter = 0;
  s->bad = a.xtoff[0] != 0u || a.xtoff[a.n] != m;
  s->done = max_iter <= 0 || s->bad;   // no sweep reads a bad CSR
  s->max_iter = max_iter;
  s->tol = tol;
}

__global__ void k_na_init(NaArgs a) {
  const double r0 = 1.0 / (double)a.n;
  double* r = a.rank(0);
  double* c = a.contrib(0);
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
    r[v] = r0;
    c[v] = r0 / (double)a.xtdat[v];
  }
}

__device__ __forceinline__ unsigned long long na_finish(const NaArgs& a, uint32_t v, double cv, int p) {
  const double rv = a.rank(p)[v];
  const double av = fma(a.P, cv, a.C0);
  a.rank(p ^ 1)[v] = av;
  a.contrib(p ^ 1)[v] = av / (double)a.xtdat[v];
  return prx::dbits(fabs(av - rv));
}

// in-degree <= 64: one thread per vertex, front to back
__global__ void __launch_bounds__(256) k_na_update_thread(NaArgs a) {
  NaState* s = a.st();
  if (s->done) return;
  const int p = s->iter & 1;
  const double* __restrict__ c = a.contrib(p);
  unsigned long long emax = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < a.n; v += gridDim.x * blockDim.x) {
    const uint32_t b = a.xtoff[v], e = a.xtoff[v + 1];
    if (e - b > prx::kLowMax) continue;
    double acc = 0.0;
    for (uint32_t j = b; j < e; ++j) acc += c[a.xtedg[j]];
    const unsigned long long ev = na_finish(a, v, acc, p);
    emax = ev > emax ? ev : emax;
  }
  prx::block_max_bits(emax, &s->el_bits[p]);
}

// in-degree > 64: one warp per vertex emulating the 256 strided partial sums
// and the halving tree
__global__ void __launch_bounds__(256) k_na_update_warp(NaArgs a) {
  NaState* s = a.st();
  if (s->done) return;
  const int p = s->iter & 1;
  const double* __restrict__ c = a.contrib(p);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long emax = 0;
  for (uint32_t v = warp; v < a.n; v += nwarps) {
    const uint32_t b = a.xtoff[v], d = a.xtoff[v + 1] - b;
    if (d <= prx::kLowMax) continue;
    double ps[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) ps[k] = 0.0;
    for (uint32_t base = 0; base < d; base += 256) {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const uint32_t t = base + lane + 32u * k;
        ps[k] += t < d ? c[a.xtedg[b + t]] : 0.0;
      }
    }
    ps[0] += ps[4]; ps[1] += ps[5]; ps[2] += ps[6]; ps[3] += ps[7];
    ps[0] += ps[2]; ps[1] += ps[3];
    ps[0] += ps[1];
    double x = ps[0];
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) {
      const unsigned long long ev = na_finish(a, v, x, p);
      emax = ev > emax ? ev : emax;
    }
  }
  prx::block_max_bits(emax, &s->el_bits[p]);
}

__global__ void k_na_finalize(NaArgs a) {
  NaState* s = a.st();
  if (s->done) return;
  const int p = s->iter & 1;
  const double el = __longlong_as_double((long long)s->el_bits[p]);
  s->iter += 1;
  if (el < s->tol || s->iter >= s->max_iter) s->done = 1;
  s->el_bits[p ^ 1] = 0;
}

// Device address of the scratch array in the current context.  Looked up on
// every call: the lookup allocates nothing, and an address cached per device
// would go stale after a device reset or under another context.
int scratch_address(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    prx::set_error(std::string("prx_static_solve_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return PRX_ECUDA;
  }
  *out = static_cast<double*>(p);
  return PRX_OK;
}

}  // namespace

extern "C" int prx_static_solve_noalloc(uint32_t n, uint64_t m, const uint32_t* xtoff, const uint32_t* xtedg,
                                        const uint32_t* xtdat, double damping, double tolerance, int max_iterations,
                                        double* ranks, int* iterations, void* stream) {
  if (iterations) *iterations = 0;
  if (n > PRX_NOALLOC_MAX_VERTICES) {
    prx::set_error("prx_static_solve_noalloc: n = " + std::to_string(n) + " exceeds the scratch limit of " +
                   std::to_string(PRX_NOALLOC_MAX_VERTICES) + " vertices");
    return PRX_ERANGE;
  }
  if (m > 0xffffffffull) {
    prx::set_error("prx_static_solve_noalloc: m >= 2^32 does not fit 32-bit offsets");
    return PRX_ERANGE;
  }
  if (!(damping > 0 && damping < 1)) {
    prx::set_error("prx_static_solve_noalloc: damping must be in (0, 1)");
    return PRX_EINVAL;
  }
  if (n == 0) return PRX_OK;
  if (!xtoff || !xtdat || !ranks || (m && !xtedg)) {
    prx::set_error("prx_static_solve_noalloc: NULL graph or ranks pointer");
    return PRX_EINVAL;
  }
  double* scratch = nullptr;
  int st = scratch_address(&scratch);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int sms = 152;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  NaArgs a;
  a.xtoff = xtoff;
  a.xtedg = xtedg;
  a.xtdat = xtdat;
  a.out = ranks;
  a.scratch = scratch;
  a.n = n;
  a.P = damping;
  a.C0 = (1 - damping) / (double)n;
  const uint32_t tgrid = (n + 255) / 256 < (uint32_t)sms * 8 ? (n + 255) / 256 : (uint32_t)sms * 8;
  k_na_reset<<<1, 1, 0, s>>>(a, (uint32_t)m, max_iterations, tolerance);
  k_na_init<<<tgrid, 256, 0, s>>>(a);
  NaState h;  // read back on the host stack; no allocation
  for (int k = 1;; k = k < 16 ? 2 * k : 16) {
    for (int i = 0; i < k; ++i) {
      k_na_update_thread<<<tgrid, 256, 0, s>>>(a);
      k_na_update_warp<<<sms * 4, 256, 0, s>>>(a);
      k_na_finalize<<<1, 1, 0, s>>>(a);
    }
    cudaError_t e = cudaMemcpyAsync(&h, scratch, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      prx::set_error(std::string("prx_static_solve_noalloc: ") + cudaGetErrorString(e));
      return PRX_ECUDA;
    }
    if (h.done) break;
  }
  if (h.bad) {
    prx::set_error("prx_static_solve_noalloc: xtoff[0] must be 0 and xtoff[n] must equal m");
    return PRX_EINVAL;
  }
  if (h.iter & 1) {  // the last sweep wrote the scratch rank buffer
    cudaError_t e = cudaMemcpyAsync(ranks, scratch + kHeadDoubles, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      prx::set_error(std::string("prx_static_solve_noalloc: ") + cudaGetErrorString(e));
      return PRX_ECUDA;
    }
  }
  if (iterations) *iterations = h.iter;
  return PRX_OK;
}
