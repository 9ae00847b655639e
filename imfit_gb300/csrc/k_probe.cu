// k_probe.cu -- measured SFU (MUFU) throughput of this GPU, for the
// per-unit roofline T_roof = B / BW_HBM + F / P_SFU of the statistic+gradient
// evaluation (F = the transcendental operations the pixel passes must issue).
//
// Every thread keeps eight independent lg2.approx -> ex2.approx chains (x -> 2^log2(x)
// stays at 1 for x near 1), so the MUFU pipe, not a dependency, sets the rate;
// the grid fills every SM at full occupancy.  Timed with CUDA events on a
// private stream, best of three after a warm-up; the clocks are whatever the
// GPU runs at (nothing is locked or changed).
#include <cuda_runtime.h>

#include "imfit_gb300.h"

namespace {

__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_sfu_rate(float *out, int iters) {
  float x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) x[k] = 1.0f + 1e-3f * (float)k + 1e-7f * (float)threadIdx.x;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = ex2_approx(lg2_approx(x[k]));
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int imfit_MeasureSfuRate(int device, double *opsPerSecond) {
  if (!opsPerSecond) return IMFIT_E_ARG;
  *opsPerSecond = 0.0;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) return IMFIT_E_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return IMFIT_E_CUDA;
  int sms = 0, perSm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_sfu_rate, kThreads, 0);
  if (sms <= 0 || perSm <= 0) {
    cudaSetDevice(prev);
    return IMFIT_E_CUDA;
  }
  const int blocks = sms * perSm, iters = 4096;
  float *out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int status = IMFIT_OK;
  float best = 0.f;
  if (cudaMalloc(&out, sizeof(float) * (size_t)blocks * kThreads) != cudaSuccess ||
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    status = IMFIT_E_CUDA;
  } else {
    k_sfu_rate<<<blocks, kThreads, 0, st>>>(out, iters);  // warm-up
    for (int r = 0; r < 3 && status == IMFIT_OK; r++) {
      cudaEventRecord(e0, st);
      k_sfu_rate<<<blocks, kThreads, 0, st>>>(out, iters);
      cudaEventRecord(e1, st);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        status = IMFIT_E_CUDA;
      else if (best == 0.f || ms < best)
        best = ms;
    }
  }
  if (status == IMFIT_OK && best > 0.f)
    *opsPerSecond = (double)blocks * kThreads * (double)iters * (2.0 * kChains) / (best * 1e-3);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  cudaSetDevice(prev);
  return status;
}
