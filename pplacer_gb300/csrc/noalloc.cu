// Allocation-free ten_log_like3 on device buffers.
//
// Some callers cannot allocate device memory at the point where they need a
// likelihood: code running inside another runtime that owns the GPU's memory
// through its own pool, or pipelines that allocate only at start-up and
// forbid cudaMalloc / cudaFree afterwards (they would synchronise the device
// and can fail under memory pressure).  This entry point serves them: the
// caller passes device pointers for the inputs and the one-double output, and
// the scratch the reduction needs -- one partial log sum per block of 256
// sites -- lives in one file-scope __device__ array of fixed size, which
// every GPU that loads this library holds until the process exits.  Nothing
// here calls cudaMalloc, cudaFree or an allocating library routine.
//
// Limits and sharing: at most kMaxSites sites per call (kMaxBlocks partial
// sums of 256 sites); every call on a device uses the same array, so calls
// that overlap on the GPU (different streams, or concurrent host threads)
// race and must be serialised by the caller.  The array keeps the last
// call's contents; every value a call reads was written earlier in that same
// call, so nothing needs clearing.  The first call on a device (and the first
// call after that device's primary context was reset, e.g. by
// cudaDeviceReset) looks up the array's device address with
// cudaGetSymbolAddress, with that device current; make that first call
// before any stream capture.
#include <math.h>

#include <cuda.h>

#include <mutex>

#include "pgb_common.cuh"

namespace pgb {
namespace {

constexpr int kThreadsNA = 256;                 // sites per block
constexpr int kMaxBlocks = 256;                 // partial sums the scratch holds
constexpr int kMaxSites = kThreadsNA * kMaxBlocks;  // 65,536 sites per call
constexpr int kMaxDevices = 64;

// one partial log sum per block of kThreadsNA sites
static __device__ __align__(256) double g_noalloc_scratch[kMaxBlocks];

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

std::mutex g_na_mu;
double *g_na_ptr[kMaxDevices] = {};
unsigned long long g_na_ctx_id[kMaxDevices] = {};  // the context each cached address belongs to
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Driver entry points looked up through the runtime (no link to libcuda).
bool driver_entry(const char *name, void **fn) {
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q);
  return e == cudaSuccess && q == cudaDriverEntryPointSuccess && *fn;
}

// Unique id of the calling thread's current context (0: none current).
bool current_context_id(unsigned long long *id) {
  CUcontext ctx = nullptr;
  *id = 0;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return false;
  return !ctx || g_ctx_get_id(ctx, id) == CUDA_SUCCESS;
}

// per-site likelihood sum_r sum_k statd_k x y z, and the block's partial sum
// of its logs (linear_c.c:367-424); one site per thread
__global__ void k_na_sites(const double *__restrict__ statd, const double *__restrict__ x,
                           const double *__restrict__ y, const double *__restrict__ z, int n_rates, int n_sites,
                           int K, double *part) {
  double acc = 0;
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n_sites) {
    double u = 0;
    for (int r = 0; r < n_rates; r++) {
      long o = ((long)r * n_sites + s) * K;
      for (int k = 0; k < K; k++) u += statd[k] * x[o + k] * y[o + k] * z[o + k];
    }
    acc = log(u);
  }
  __shared__ double sh[kThreadsNA / 32];
  acc = warp_sum_d(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int i = 0; i < kThreadsNA / 32; i++) t += sh[i];
    part[blockIdx.x] = t;
  }
}

// ordered sum of the partials, minus n_sites log(n_rates) as linear_c.c:421
__global__ void k_na_finish(const double *part, int n_parts, int n_sites, int n_rates, double *result) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t = 0;
  for (int i = 0; i < n_parts; i++) t += part[i];
  *result = t - ((double)(float)n_sites) * log((double)(float)n_rates);
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" pgb_status pgb_ten_log_like3_noalloc(const double *statd, const double *x, const double *y,
                                                const double *z, int n_rates, int n_sites, int n_states,
                                                double *result, void *stream) {
  if (!statd || !x || !y || !z || !result || n_rates < 1 || n_states < 1 || n_sites < 1) {
    set_error("ten_log_like3_noalloc: null pointer or empty size");
    return PGB_ERR_ARG;
  }
  if (n_sites > kMaxSites) {
    set_error("ten_log_like3_noalloc: %d sites exceed the fixed scratch of %d sites", n_sites, kMaxSites);
    return PGB_ERR_ARG;
  }
  int dev = 0;
  PGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("ten_log_like3_noalloc: device %d beyond the supported %d", dev, kMaxDevices);
    return PGB_ERR_ARG;
  }
  double *scratch;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_ctx_get_current || !g_ctx_get_id) {
      void *f1 = nullptr, *f2 = nullptr;
      if (!driver_entry("cuCtxGetCurrent", &f1) || !driver_entry("cuCtxGetId", &f2)) {
        set_error("ten_log_like3_noalloc: driver context entry points unavailable");
        return PGB_ERR_CUDA;
      }
      g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
      g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    unsigned long long id = 0;
    if (!current_context_id(&id)) {
      set_error("ten_log_like3_noalloc: cannot read the current context");
      return PGB_ERR_CUDA;
    }
    // Once per device and context (a reset device gets a new context, into
    // which the library's module, and so the array, is loaded afresh), with
    // that device current.  cudaGetSymbolAddress also makes the device's
    // primary context current where no context is.
    if (id == 0 || !g_na_ptr[dev] || g_na_ctx_id[dev] != id) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        set_error("ten_log_like3_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return PGB_ERR_CUDA;
      }
      if (!current_context_id(&id) || id == 0) {
        set_error("ten_log_like3_noalloc: no current context on device %d", dev);
        return PGB_ERR_CUDA;
      }
      g_na_ptr[dev] = static_cast<double *>(p);
      g_na_ctx_id[dev] = id;
    }
    scratch = g_na_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int blocks = (n_sites + kThreadsNA - 1) / kThreadsNA;  // <= kMaxBlocks by the size check
  k_na_sites<<<blocks, kThreadsNA, 0, st>>>(statd, x, y, z, n_rates, n_sites, n_states, scratch);
  PGB_LAUNCH_CHECK();
  k_na_finish<<<1, 32, 0, st>>>(scratch, blocks, n_sites, n_rates, result);
  PGB_LAUNCH_CHECK();
  return PGB_OK;
}
