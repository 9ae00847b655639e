// psf_interp.cuh -- PSF interpolation for the PointSource functions
// (function_objects/psf_interpolators.cpp, func_pointsource.cpp,
// func_pointsource-rot.cpp).
//
// The PSF's pixel centres sit at offsets k - (N-1)/2 from its centre; the
// interpolant is zero outside [-(N-1)/2, (N-1)/2] in either axis
// (psf_interpolators.cpp:82-92).
//
// Bicubic: the reference calls GSL's gsl_interp2d_bicubic.  Its published
// method -- partial derivatives z_x, z_y, z_xy at every grid point from natural
// cubic splines through the grid lines, and in each cell the bicubic Hermite
// patch matching z, z_x, z_y, z_xy at the four corners (a point on an interior
// grid line belongs to the cell on its positive side, the last line to the
// cell before it) -- is restated here; the four tables are built once on the
// host in FP64 (psf_interp_tables in model_object.cpp).
//
// Lanczos2/3 (psf_interpolators.cpp:139-300): sum over the (2n+1)^2 samples
// around floor(x + (N-1)/2), weight Lanczos(dx) Lanczos(dy), the PSF read as
// data[ix * nColumns + iy] (x index first, as the reference indexes it).
#pragma once
#include <cuda_runtime.h>

namespace imfit {

enum PsfInterpKind : int { PSF_BICUBIC = 1, PSF_LANCZOS2 = 2, PSF_LANCZOS3 = 3 };

// t: bicubic -> 4 planes of nc*nr values (z, z_x, z_y, z_xy; row-major, x
// fastest); Lanczos -> the PSF itself (row-major).
template <typename T>
struct PsfInterp {
  int kind, nc, nr, pad;
  T xb, yb;
  const T *t;
};

// Cubic Hermite weights on [0,1]: values at the two ends (h0, h1) and slopes
// at the two ends (g0, g1), with their t-derivatives.
template <typename T>
__host__ __device__ inline void hermite_w(T t, T &h0, T &h1, T &g0, T &g1) {
  const T t2 = t * t, t3 = t2 * t;
  h0 = (T)2 * t3 - (T)3 * t2 + (T)1;
  h1 = (T)-2 * t3 + (T)3 * t2;
  g0 = t3 - (T)2 * t2 + t;
  g1 = t3 - t2;
}
template <typename T>
__host__ __device__ inline void hermite_dw(T t, T &h0, T &h1, T &g0, T &g1) {
  const T t2 = t * t;
  h0 = (T)6 * t2 - (T)6 * t;
  h1 = (T)-6 * t2 + (T)6 * t;
  g0 = (T)3 * t2 - (T)4 * t + (T)1;
  g1 = (T)3 * t2 - (T)2 * t;
}

// Lanczos kernel (psf_interpolators.cpp:299-309), with the reference's PI
// constants; FP64.
__host__ __device__ inline double lanczos64(double x, int n) {
  const double pi = 3.14159265358979, pi2 = 9.86960440108936;
  const double a = fabs(x);
  if (a < 1.0e-6) return 1.0;
  if (a > n) return 0.0;
  return (n * sin(pi * a) * sin(pi * a / n)) / (pi2 * a * a);
}

// bicubic cell and local coordinates; false outside the PSF's extent
template <typename T>
__host__ __device__ inline bool bicubic_cell(const PsfInterp<T> &ip, T x, T y, int &i, int &j, T &t, T &u) {
  if (x < -ip.xb || x > ip.xb || y < -ip.yb || y > ip.yb) return false;
  i = (int)floor(x + ip.xb);
  j = (int)floor(y + ip.yb);
  if (i > ip.nc - 2) i = ip.nc - 2;
  if (j > ip.nr - 2) j = ip.nr - 2;
  if (i < 0) i = 0;
  if (j < 0) j = 0;
  t = x - ((T)i - ip.xb);
  u = y - ((T)j - ip.yb);
  return true;
}

// PsfInterpolator::GetValue, FP64 (plain path)
__host__ __device__ inline double psf_interp64(const PsfInterp<double> &ip, double x, double y) {
  if (ip.kind == PSF_BICUBIC) {
    int i, j;
    double t, u;
    if (!bicubic_cell(ip, x, y, i, j, t, u)) return 0.0;
    double a0, a1, b0, b1, c0, c1, e0, e1;
    hermite_w(t, a0, a1, b0, b1);
    hermite_w(u, c0, c1, e0, e1);
    const long np = (long)ip.nc * ip.nr;
    const double *z = ip.t, *zx = z + np, *zy = zx + np, *zxy = zy + np;
    const long k00 = (long)j * ip.nc + i, k10 = k00 + 1, k01 = k00 + ip.nc, k11 = k01 + 1;
    double v = 0.0;
    v += z[k00] * a0 * c0 + z[k10] * a1 * c0 + z[k01] * a0 * c1 + z[k11] * a1 * c1;
    v += zx[k00] * b0 * c0 + zx[k10] * b1 * c0 + zx[k01] * b0 * c1 + zx[k11] * b1 * c1;
    v += zy[k00] * a0 * e0 + zy[k10] * a1 * e0 + zy[k01] * a0 * e1 + zy[k11] * a1 * e1;
    v += zxy[k00] * b0 * e0 + zxy[k10] * b1 * e0 + zxy[k01] * b0 * e1 + zxy[k11] * b1 * e1;
    return v;
  }
  if (x < -ip.xb || x > ip.xb || y < -ip.yb || y > ip.yb) return 0.0;
  const int n = (ip.kind == PSF_LANCZOS2) ? 2 : 3;
  const int imx = (int)floor(x + ip.xb), imy = (int)floor(y + ip.yb);
  double v = 0.0;
  for (int a = -n; a <= n; a++) {
    const int ix = imx + a;
    if (ix < 0 || ix >= ip.nc) continue;
    const double xd = ix - ip.xb;
    for (int b = -n; b <= n; b++) {
      const int iy = imy + b;
      if (iy < 0 || iy >= ip.nr) continue;
      const double yd = iy - ip.yb;
      v += lanczos64(x - xd, n) * lanczos64(y - yd, n) * ip.t[(long)ix * ip.nc + iy];
    }
  }
  return v;
}

#ifdef __CUDACC__
// Lanczos kernel and its derivative, FP32 (fast path)
__device__ inline void lanczos32(float x, int n, float &L, float &dL) {
  const float a = fabsf(x);
  if (a < 1.0e-6f) {
    L = 1.f;
    dL = 0.f;
    return;
  }
  if (a > (float)n) {
    L = dL = 0.f;
    return;
  }
  const float inv_n = n == 2 ? 0.5f : 0.33333333f;
  float s1, c1, s2, c2;
  sincospif(a, &s1, &c1);
  sincospif(a * inv_n, &s2, &c2);
  const float pi = 3.14159265f, inv_pi2 = 0.10132118f;  // 1/pi^2
  const float ia = __frcp_rn(a);
  const float f = s1 * s2;
  L = (float)n * f * inv_pi2 * ia * ia;
  const float df = pi * (c1 * s2 + inv_n * s1 * c2);
  const float dLa = (float)n * inv_pi2 * (df * ia * ia - 2.f * f * ia * ia * ia);
  dL = x < 0.f ? -dLa : dLa;
}

// value and partial derivatives of the interpolant, FP32
__device__ inline void psf_interp32(const PsfInterp<float> &ip, float x, float y, float &v, float &vx, float &vy) {
  v = vx = vy = 0.f;
  if (ip.kind == PSF_BICUBIC) {
    int i, j;
    float t, u;
    if (!bicubic_cell(ip, x, y, i, j, t, u)) return;
    float a0, a1, b0, b1, c0, c1, e0, e1, da0, da1, db0, db1, dc0, dc1, de0, de1;
    hermite_w(t, a0, a1, b0, b1);
    hermite_w(u, c0, c1, e0, e1);
    hermite_dw(t, da0, da1, db0, db1);
    hermite_dw(u, dc0, dc1, de0, de1);
    const long np = (long)ip.nc * ip.nr;
    const float *z = ip.t, *zx = z + np, *zy = zx + np, *zxy = zy + np;
    const long k00 = (long)j * ip.nc + i, k10 = k00 + 1, k01 = k00 + ip.nc, k11 = k01 + 1;
    const float Z[4] = {__ldg(z + k00), __ldg(z + k10), __ldg(z + k01), __ldg(z + k11)};
    const float X[4] = {__ldg(zx + k00), __ldg(zx + k10), __ldg(zx + k01), __ldg(zx + k11)};
    const float Y[4] = {__ldg(zy + k00), __ldg(zy + k10), __ldg(zy + k01), __ldg(zy + k11)};
    const float W[4] = {__ldg(zxy + k00), __ldg(zxy + k10), __ldg(zxy + k01), __ldg(zxy + k11)};
    // per corner: x-weights (value, slope) and y-weights (value, slope)
    const float hx[4] = {a0, a1, a0, a1}, gx[4] = {b0, b1, b0, b1};
    const float hy[4] = {c0, c0, c1, c1}, gy[4] = {e0, e0, e1, e1};
    const float dhx[4] = {da0, da1, da0, da1}, dgx[4] = {db0, db1, db0, db1};
    const float dhy[4] = {dc0, dc0, dc1, dc1}, dgy[4] = {de0, de0, de1, de1};
#pragma unroll
    for (int c = 0; c < 4; c++) {
      v += Z[c] * hx[c] * hy[c] + X[c] * gx[c] * hy[c] + Y[c] * hx[c] * gy[c] + W[c] * gx[c] * gy[c];
      vx += Z[c] * dhx[c] * hy[c] + X[c] * dgx[c] * hy[c] + Y[c] * dhx[c] * gy[c] + W[c] * dgx[c] * gy[c];
      vy += Z[c] * hx[c] * dhy[c] + X[c] * gx[c] * dhy[c] + Y[c] * hx[c] * dgy[c] + W[c] * gx[c] * dgy[c];
    }
    return;
  }
  if (x < -ip.xb || x > ip.xb || y < -ip.yb || y > ip.yb) return;
  const int n = (ip.kind == PSF_LANCZOS2) ? 2 : 3;
  const int imx = (int)floorf(x + ip.xb), imy = (int)floorf(y + ip.yb);
  float Ly[7], dLy[7];
  for (int b = -n; b <= n; b++) lanczos32(y - ((float)(imy + b) - ip.yb), n, Ly[b + n], dLy[b + n]);
  for (int a = -n; a <= n; a++) {
    const int ix = imx + a;
    if (ix < 0 || ix >= ip.nc) continue;
    float Lx, dLx;
    lanczos32(x - ((float)ix - ip.xb), n, Lx, dLx);
    for (int b = -n; b <= n; b++) {
      const int iy = imy + b;
      if (iy < 0 || iy >= ip.nr) continue;
      const float d = __ldg(ip.t + (long)ix * ip.nc + iy);
      v += Lx * Ly[b + n] * d;
      vx += dLx * Ly[b + n] * d;
      vy += Lx * dLy[b + n] * d;
    }
  }
}
#endif

}  // namespace imfit
