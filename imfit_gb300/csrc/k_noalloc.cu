// k_noalloc.cu -- chi^2 of device-resident arrays without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need a fit
// statistic: a plug-in running inside a host framework that reserves all
// device memory up front and forbids its plug-ins to call the allocator, an
// embedded deployment whose device-memory budget is fixed at start-up, or a
// latency-critical solver loop that must not take the allocator's locks or
// trigger the implicit device synchronisation that cudaFree performs.  For
// them, imfit_ChiSquaredDeviceNoAlloc
// runs the same two-level enorm reduction as the plain chi^2 kernel, but keeps
// its per-block partial sums in a fixed, file-scope __device__ array instead
// of a buffer from cudaMalloc.  The caller passes only its inputs and the
// output pointer.
//
// Compiled with --fmad=false, like the plain FP64 kernels, so the arithmetic
// matches them term for term.
#include <cuda.h>  // CUcontext / CUresult types; driver calls go through cudaGetDriverEntryPointByVersion

#include <cstdio>
#include <mutex>

#include "../../include/imfit_gb300.h"
#include "stat_common.cuh"

namespace imfit {
void set_global_error(const char *msg);
}

namespace {

using namespace imfit;

constexpr int kThreads = 256;
constexpr int kTermsPerThread = 8;
constexpr long kTermsPerBlock = (long)kThreads * kTermsPerThread;

// Partial enorm states, 5 doubles per block: 4096 blocks, 160 KiB.  Every GPU
// that loads this library holds the array until the process exits.
static __device__ __align__(256) double g_noalloc_partials[IMFIT_NOALLOC_MAX_BLOCKS * 5];

__global__ void __launch_bounds__(kThreads) k_chi2_noalloc_partial(const double *__restrict__ model,
                                                                   const double *__restrict__ data,
                                                                   const double *__restrict__ weight, long n,
                                                                   double *__restrict__ partials) {
  Enorm e = {0, 0, 0, 0, 0};
  const double agiant = 1.304e19 / (double)(int)n;
  const long base = blockIdx.x * kTermsPerBlock;
  for (int k = 0; k < kTermsPerThread; k++) {
    const long z = base + (long)k * kThreads + threadIdx.x;
    if (z < n) enorm_add(e, weight[z] * (data[z] - model[z]), agiant);
  }
  e = block_enorm(e);
  if (threadIdx.x == 0) {
    double *p = partials + blockIdx.x * 5;
    p[0] = e.s1;
    p[1] = e.x1;
    p[2] = e.s2;
    p[3] = e.s3;
    p[4] = e.x3;
  }
}

__global__ void __launch_bounds__(kThreads) k_chi2_noalloc_final(const double *__restrict__ partials, int nPart,
                                                                 double *__restrict__ result) {
  Enorm e = {0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < nPart; i += blockDim.x) {
    const double *p = partials + i * 5;
    Enorm o = {p[0], p[1], p[2], p[3], p[4]};
    enorm_merge(e, o);
  }
  e = block_enorm(e);
  if (threadIdx.x == 0) {
    const double chi = enorm_final(e);
    *result = chi * chi;
  }
}

// Device address of g_noalloc_partials, looked up with cudaGetSymbolAddress
// once per CUDA context (with its device current) and cached under the
// context's driver-assigned ID.  In host code the symbol itself is only a
// host-side handle.  The ID is unique for the life of the process, so a
// context re-created after cudaDeviceReset, or a caller's own driver-API
// context on the same device, gets a fresh lookup instead of a stale address.
// Where the driver's context queries are unavailable the cache falls back to
// the device ordinal.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

struct ScratchSlot {
  unsigned long long ctx;  // context ID (or ordinal + 1 in the fallback)
  double *ptr;
};
constexpr int kMaxSlots = 64;
std::mutex g_lock;
ScratchSlot g_slots[kMaxSlots] = {};
int g_nextSlot = 0;
bool g_triedDriver = false;
CtxGetCurrentFn g_getCurrent = nullptr;
CtxGetIdFn g_getId = nullptr;

// caller holds g_lock
bool context_key(unsigned long long *key) {
  if (!g_triedDriver) {
    g_triedDriver = true;
    cudaDriverEntryPointQueryResult q;
    void *f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_getCurrent = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_getId = reinterpret_cast<CtxGetIdFn>(f);
  }
  if (!g_getCurrent || !g_getId) return false;
  CUcontext c = nullptr;
  if (g_getCurrent(&c) != CUDA_SUCCESS || !c) return false;
  unsigned long long id = 0;
  if (g_getId(c, &id) != CUDA_SUCCESS) return false;
  *key = id | (1ull << 63);  // disjoint from the ordinal keys
  return true;
}

cudaError_t scratch_for_current_context(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e) return e;
  std::lock_guard<std::mutex> g(g_lock);
  unsigned long long key = 0;
  bool haveKey = context_key(&key);
  if (haveKey) {
    for (const ScratchSlot &s : g_slots)
      if (s.ptr && s.ctx == key) {
        *out = s.ptr;
        return cudaSuccess;
      }
  }
  void *p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_partials);  // also makes the device's context current
  if (e) return e;
  if (!haveKey && !context_key(&key)) key = (unsigned long long)dev + 1;
  if (!haveKey && key == (unsigned long long)dev + 1) {
    // fallback keyed by ordinal: reuse this device's slot
    for (ScratchSlot &s : g_slots)
      if (s.ptr && s.ctx == key) {
        s.ptr = static_cast<double *>(p);
        *out = s.ptr;
        return cudaSuccess;
      }
  }
  ScratchSlot &s = g_slots[g_nextSlot];
  g_nextSlot = (g_nextSlot + 1) % kMaxSlots;
  s.ctx = key;
  s.ptr = static_cast<double *>(p);
  *out = s.ptr;
  return cudaSuccess;
}

}  // namespace

extern "C" int imfit_ChiSquaredDeviceNoAlloc(const double *d_model, const double *d_data,
                                             const double *d_weight, long nPixels, double *d_result,
                                             void *stream) {
  if (!d_model || !d_data || !d_weight || !d_result || nPixels < 1) {
    set_global_error("ChiSquaredDeviceNoAlloc: null pointer or empty input");
    return IMFIT_E_ARG;
  }
  const long maxPixels = (long)IMFIT_NOALLOC_MAX_BLOCKS * kTermsPerBlock;
  if (nPixels > maxPixels) {
    char msg[160];
    snprintf(msg, sizeof msg, "ChiSquaredDeviceNoAlloc: %ld pixels exceed the fixed scratch limit of %ld",
             nPixels, maxPixels);
    set_global_error(msg);
    return IMFIT_E_ARG;
  }
  double *scratch = nullptr;
  cudaError_t e = scratch_for_current_context(&scratch);
  if (e) {
    set_global_error(cudaGetErrorString(e));
    return IMFIT_E_CUDA;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // every partial slot the final kernel reads is written by this call's first
  // kernel, so no clearing of the shared array is needed
  const int nBlocks = (int)((nPixels + kTermsPerBlock - 1) / kTermsPerBlock);
  k_chi2_noalloc_partial<<<nBlocks, kThreads, 0, st>>>(d_model, d_data, d_weight, nPixels, scratch);
  k_chi2_noalloc_final<<<1, kThreads, 0, st>>>(scratch, nBlocks, d_result);
  e = cudaGetLastError();
  if (e) {
    set_global_error(cudaGetErrorString(e));
    return IMFIT_E_CUDA;
  }
  return 0;
}
