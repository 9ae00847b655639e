// stat_common.cuh -- device helpers shared by the FP64 statistic kernels:
// the MINPACK enorm accumulator as a mergeable state and block reductions.
#pragma once
#include <cuda_runtime.h>

namespace imfit {

// MINPACK enorm (core/mp_enorm.cpp:51-122) as a mergeable state: sums of
// squares of large / intermediate / small magnitudes, the first and last
// kept scaled by their running maxima.
struct Enorm {
  double s1, x1, s2, s3, x3;
};

__device__ __forceinline__ void enorm_add(Enorm &e, double v, double agiant) {
  const double rdwarf = 3.834e-20;
  const double xabs = fabs(v);
  if (xabs > rdwarf && xabs < agiant) {
    e.s2 += xabs * xabs;
  } else if (xabs > rdwarf) {
    if (xabs > e.x1) {
      const double t = e.x1 / xabs;
      e.s1 = 1.0 + e.s1 * t * t;
      e.x1 = xabs;
    } else {
      const double t = xabs / e.x1;
      e.s1 += t * t;
    }
  } else if (xabs > e.x3) {
    const double t = e.x3 / xabs;
    e.s3 = 1.0 + e.s3 * t * t;
    e.x3 = xabs;
  } else if (xabs != 0.0) {
    const double t = xabs / e.x3;
    e.s3 += t * t;
  }
}

__device__ __forceinline__ void scaled_merge(double &s, double &x, double s2, double x2) {
  if (x2 > x) {
    const double t = x / x2;
    s = s2 + s * t * t;
    x = x2;
  } else if (x2 > 0.0) {
    const double t = x2 / x;
    s += s2 * t * t;
  }
}

__device__ __forceinline__ void enorm_merge(Enorm &a, const Enorm &b) {
  scaled_merge(a.s1, a.x1, b.s1, b.x1);
  a.s2 += b.s2;
  scaled_merge(a.s3, a.x3, b.s3, b.x3);
}

__device__ __forceinline__ double enorm_final(const Enorm &e) {
  if (e.s1 != 0.0) return e.x1 * sqrt(e.s1 + (e.s2 / e.x1) / e.x1);
  if (e.s2 != 0.0) {
    double temp;
    if (e.s2 >= e.x3)
      temp = e.s2 * (1.0 + (e.x3 / e.s2) * (e.x3 * e.s3));
    else
      temp = e.x3 * ((e.s2 / e.x3) + (e.x3 * e.s3));
    return sqrt(temp);
  }
  return e.x3 * sqrt(e.s3);
}

__device__ __forceinline__ Enorm enorm_shfl(const Enorm &e, int off) {
  Enorm o;
  o.s1 = __shfl_down_sync(0xffffffffu, e.s1, off);
  o.x1 = __shfl_down_sync(0xffffffffu, e.x1, off);
  o.s2 = __shfl_down_sync(0xffffffffu, e.s2, off);
  o.s3 = __shfl_down_sync(0xffffffffu, e.s3, off);
  o.x3 = __shfl_down_sync(0xffffffffu, e.x3, off);
  return o;
}

__device__ __forceinline__ Enorm block_enorm(Enorm e) {
  __shared__ Enorm sh[32];
  for (int off = 16; off > 0; off >>= 1) {
    Enorm o = enorm_shfl(e, off);
    enorm_merge(e, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = e;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    e = (lane < nw) ? sh[lane] : Enorm{0, 0, 0, 0, 0};
    for (int off = 16; off > 0; off >>= 1) {
      Enorm o = enorm_shfl(e, off);
      enorm_merge(e, o);
    }
  }
  return e;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[32];
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    v = (lane < nw) ? sh[lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  }
  return v;
}

}  // namespace imfit
