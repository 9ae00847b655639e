// ffsum.cuh -- double-float ("float-float") sums for the fast path's reductions.
//
// A value is carried as an unevaluated sum hi + lo of two FP32 numbers and
// added with Knuth's TwoSum (an error-free transformation: s + e equals
// a + b exactly), renormalised after every addition (Dekker's FastTwoSum).
// This keeps about 44 significant bits -- FP64-class accuracy for sums of
// FP32 terms -- while running on the FP32 pipe: on this GPU the FP64 pipe
// issues about two operations per SM per clock, so FP64 trees over every
// CTA's partials would cost more than the pixel work they sum.  Orders are
// fixed, so results are deterministic.  (No multiplications: nothing here can
// be contracted into an FMA.)
#pragma once
#include <cuda_runtime.h>

namespace imfit {

struct ffloat {
  float hi, lo;
};

__device__ __forceinline__ ffloat ff_make(float v) { return {v, 0.f}; }

// (a.hi + a.lo) + (b.hi + b.lo)
__device__ __forceinline__ ffloat ff_add(ffloat a, ffloat b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo);
  const float hi = s + e;
  return {hi, e - (hi - s)};
}

__device__ __forceinline__ ffloat ff_add(ffloat a, float b) { return ff_add(a, ffloat{b, 0.f}); }

__device__ __forceinline__ double ff_value(ffloat a) { return (double)a.hi + (double)a.lo; }

// Butterfly sum over the warp; lane 0's result is the reference value.
__device__ __forceinline__ ffloat ff_warp_sum(ffloat v) {
  for (int o = 16; o > 0; o >>= 1) {
    ffloat w;
    w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v = ff_add(v, w);
  }
  return v;
}

__device__ __forceinline__ float2 ff_store(ffloat v) { return make_float2(v.hi, v.lo); }
__device__ __forceinline__ ffloat ff_load(float2 v) { return {v.x, v.y}; }

}  // namespace imfit
