// k_los.cu -- plain FP64 line-of-sight integrals of the 3-D functions, one
// thread per (model pixel, 3-D component), QAGS per pixel (qags_dev.cuh).
// Compiled with --fmad=false like the rest of the plain path: the integrand
// and set-up expressions are evaluated in the reference's order.
//
//   ExponentialDisk3D  function_objects/func_expdisk3d.cpp:178-266
//   FerrersBar3D       function_objects/func_ferrersbar3d.cpp:172-258,
//                      Compute3dObjectCoords function_objects/helper_funcs_3d.cpp:65-82
#include "kernels.h"
#include "qags_dev.cuh"

namespace imfit {

constexpr double kCoshLimit = 100.0;       // func_expdisk3d.cpp:64
constexpr double kExpDiskIntegMult = 20.0; // func_expdisk3d.cpp:66
constexpr double kLosEpsRel = 1.0e-6;      // integrator.cpp:39-51

// LuminosityDensity of ExponentialDisk3D along the line of sight s.
struct ExpDiskLos64 {
  double x_d0, y_d0, z_d0, cosInc, sinInc, J_0, h, z_0, scaledZ0, two_to_alpha, alpha;
  __device__ double operator()(double s) const {
    double y_d = y_d0 + s * sinInc;
    double z_d = z_d0 - s * cosInc;
    double R = sqrt(x_d0 * x_d0 + y_d * y_d);
    double z = fabs(z_d);
    double vs;
    if ((z / scaledZ0) > kCoshLimit) {
      vs = two_to_alpha * exp(-z / z_0);
    } else {
      double sech = 1.0 / cosh(z / scaledZ0);
      vs = pow(sech, alpha);
    }
    return J_0 * exp(-R / h) * vs;
  }
};

// LuminosityDensity of FerrersBar3D (the reference pairs y_bar with a^2 and
// x_bar with b^2).
struct FerrersLos64 {
  double x_d0, y_d0, z_d0, cosInc, sinInc, cosB, sinB, J_0, a2, b2, c2, n;
  __device__ double operator()(double s) const {
    double y_d = y_d0 + s * sinInc;
    double z_d = z_d0 - s * cosInc;
    double x_bar = x_d0 * cosB + y_d * sinB;
    double y_bar = -x_d0 * sinB + y_d * cosB;
    double z_bar = fabs(z_d);
    double m2 = y_bar * y_bar / a2 + x_bar * x_bar / b2 + z_bar * z_bar / c2;
    if (m2 > 1.0) return 0.0;
    return J_0 * pow((1.0 - m2), n);
  }
};

// GetValue(x, y) of a 3-D component (FP64 fields as comp_setup64 fills them).
__device__ double los_value64(const CompF64 &c, double x, double y, int &status) {
  double x_diff = x - c.x0, y_diff = y - c.y0;
  double xp = x_diff * c.cosPA + y_diff * c.sinPA;
  double yp = -x_diff * c.sinPA + y_diff * c.cosPA;
  double result = 0.0;
  if (c.type == F_EXPDISK3D) {
    ExpDiskLos64 f;
    f.x_d0 = xp;
    f.y_d0 = yp * c.e;
    f.z_d0 = yp * c.f;
    f.cosInc = c.e;
    f.sinInc = c.f;
    f.J_0 = c.a;
    f.h = c.b;
    f.z_0 = c.d;
    f.scaledZ0 = c.h;
    f.two_to_alpha = c.i;
    f.alpha = c.g;
    const double lim = kExpDiskIntegMult * c.b;
    status = qags_integrate(f, -lim, lim, kLosEpsRel, result);
  } else {
    FerrersLos64 f;
    f.x_d0 = xp;
    f.y_d0 = yp * c.e;
    f.z_d0 = yp * c.f;
    f.cosInc = c.e;
    f.sinInc = c.f;
    f.cosB = c.g;
    f.sinB = c.h;
    f.J_0 = c.a;
    f.a2 = c.i;
    f.b2 = c.j;
    f.c2 = c.k;
    f.n = c.l;
    const double lim = c.m;
    status = qags_integrate(f, -lim, lim, kLosEpsRel, result);
  }
  return result;
}

// out[k3 * n + pixel]: value of the k3-th 3-D component at every model pixel.
// Pixel coordinates as in k_eval64.  *flag gets bit 0 set when an integral
// needed more subintervals than the device list holds.
__global__ void __launch_bounds__(128) k_los64(const CompF64 *__restrict__ comps, LosList64 list,
                                               double *__restrict__ out, Grid64 g, int *__restrict__ flag) {
  const long n = (long)g.nCols * g.nRows;
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const CompF64 c = comps[list.comp[blockIdx.y]];
  const long j = k % g.nCols, i = k / g.nCols;
  double x, y;
  if (!g.isRegion) {
    y = (double)(i - g.pr + 1);
    x = (double)(j - g.pc + 1);
  } else {
    y = g.y1 + g.off + (i - g.pr) * g.frac;
    x = g.x1 + g.off + (j - g.pc) * g.frac;
  }
  int status = 0;
  out[(long)blockIdx.y * n + k] = los_value64(c, x, y, status);
  if (status == kQagsCapped) atomicOr(flag, 1);
}

cudaError_t launch_los64(const CompF64 *comps, const LosList64 &list, double *out, Grid64 g, int *flag,
                         cudaStream_t st) {
  const long n = (long)g.nCols * g.nRows;
  if (n == 0 || list.n == 0) return cudaSuccess;
  k_los64<<<dim3((unsigned)((n + 127) / 128), list.n), 128, 0, st>>>(comps, list, out, g, flag);
  return cudaGetLastError();
}

}  // namespace imfit

namespace imfit {

// FindTotalFluxes' grid integration (core/model_object.cpp:2415-2470): the sum
// of one component's GetValue over an xSize x ySize image with IRAF pixel
// centres (x = j+1, y = i+1).  Grid-stride over pixels, one FP64 partial per
// block (tree reduction in a fixed order); the host adds the partials.
__global__ void __launch_bounds__(256) k_flux64(CompF64 c, int xSize, int ySize, double *__restrict__ partials,
                                                int *__restrict__ flag) {
  __shared__ double red[256];
  const long n = (long)xSize * ySize;
  double acc = 0.0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const long i = k / xSize, j = k - i * xSize;
    const double x = (double)(j + 1), y = (double)(i + 1);
    if (c.type == F_EXPDISK3D || c.type == F_FERRERS3D) {
      int status = 0;
      acc += los_value64(c, x, y, status);
      if (status == kQagsCapped) atomicOr(flag, 1);
    } else {
      acc += comp_value64_2d(c, x, y);
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

cudaError_t launch_flux64(const CompF64 &c, int xSize, int ySize, double *partials, int nBlocks, int *flag,
                          cudaStream_t st) {
  k_flux64<<<nBlocks, 256, 0, st>>>(c, xSize, ySize, partials, flag);
  return cudaGetLastError();
}

}  // namespace imfit
