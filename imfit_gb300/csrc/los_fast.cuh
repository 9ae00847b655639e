// los_fast.cuh -- FP32 line-of-sight integrals of the 3-D functions for the
// fast path: one warp per (pixel, component), adaptive 21-point
// Gauss-Kronrod with lanes 0..20 evaluating the nodes of one panel, the panel
// list held one panel per lane (at most 32), global bisection of the panel
// with the largest |K21 - G10| until the sum of those differences is below
// kLosEpsRelFast of the integral.  Integrands and their analytic parameter
// derivatives:
//   ExponentialDisk3D  J_0 exp(-R/h) sech^(2/n)(n |z| / (2 z_0))    (function_objects/func_expdisk3d.cpp:226-266)
//   FerrersBar3D       J_0 (1 - m^2)^n inside the ellipsoid m^2 < 1  (function_objects/func_ferrersbar3d.cpp:230-258)
// along s with y_d = yp cos(i) + s sin(i), z_d = yp sin(i) - s cos(i).
// Initial panels: ExponentialDisk3D over [-20h, 20h] split where y_d = 0
// (the radial cusp) and where z_d = 0 (the vertical peak); FerrersBar3D over
// the exact chord of the ellipsoid (m^2 is quadratic in s), where the
// integrand is smooth, so integer n needs a single panel.  The reference's
// QAGS with epsrel 1e-6 integrates over the fixed ranges instead; both are
// integrals of the same function.  The derivative of the integration range
// (20h) is not included: the integrand is below e^-20 of its peak there.
#pragma once
#include "common.cuh"
#include "gk21_nodes.cuh"

namespace imfit {

constexpr float kLosEpsRelFast = 4e-6f;
constexpr int kLosMaxPanels = 32;
constexpr int kLosGrad = 10;  // X0, Y0 and up to 8 function parameters
constexpr float kLog2eF = 1.4426950408889634f;
constexpr float kLn2F = 0.6931471805599453f;
constexpr float kDeg2RadF = 0.017453292519943295f;

__device__ __forceinline__ float los_wsum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ------------------------------------------------------------ integrands
__device__ __forceinline__ float expdisk_f(const CompF32 &c, float xp, float yp, float s) {
  const float yd = fmaf(s, c.s4, yp * c.s3);
  const float zd = fmaf(-s, c.s3, yp * c.s4);
  const float R = fast_sqrt(fmaf(xp, xp, yd * yd));
  const float u = fabsf(zd) * c.s6;
  const float e2u = fast_ex2(-2.f * kLog2eF * u);
  // log2 sech^alpha(u) = alpha (1 - u log2 e - log2(1 + e^-2u))
  const float l2V = c.s5 * (1.f - u * kLog2eF - fast_lg2(1.f + e2u));
  return c.s0 * fast_ex2(fmaf(-R * c.s1, kLog2eF, l2V));
}

// value and d/d(X0, Y0, PA, inc, J_0, h, n, z_0)
__device__ __forceinline__ float expdisk_fg(const CompF32 &c, float xp, float yp, float s, float *g) {
  const float ci = c.s3, si = c.s4;
  const float yd = fmaf(s, si, yp * ci);
  const float zd = fmaf(-s, ci, yp * si);
  const float R = fast_sqrt(fmaf(xp, xp, yd * yd));
  const float Rinv = R > 0.f ? __fdividef(1.f, R) : 0.f;
  const float u = fabsf(zd) * c.s6;
  const float e2u = fast_ex2(-2.f * kLog2eF * u);
  const float th = __fdividef(1.f - e2u, 1.f + e2u);  // tanh(u)
  const float l1p = fast_lg2(1.f + e2u);
  const float alpha = c.s5;
  const float E = fast_ex2(fmaf(-R * c.s1, kLog2eF, alpha * (1.f - u * kLog2eF - l1p)));
  const float f = c.s0 * E;
  const float fR = -f * c.s1;
  const float fxp = fR * xp * Rinv;
  const float fyd = fR * yd * Rinv;
  const float sgn = zd > 0.f ? 1.f : (zd < 0.f ? -1.f : 0.f);
  const float iz0 = c.s6 * c.s5;  // 1/z_0 = alpha / (alpha z_0)
  const float fzd = -f * th * sgn * iz0;
  const float gp = fmaf(fyd, ci, fzd * si);
  g[0] = fmaf(-c.cosPA, fxp, c.sinPA * gp);
  g[1] = fmaf(-c.sinPA, fxp, -c.cosPA * gp);
  g[2] = kDeg2RadF * fmaf(fxp, yp, -gp * xp);
  g[3] = kDeg2RadF * fmaf(fyd, fmaf(s, ci, -yp * si), fzd * fmaf(yp, ci, s * si));
  g[4] = E;
  g[5] = f * R * c.s1 * c.s1;
  const float lncosh = (u * kLog2eF + l1p - 1.f) * kLn2F;
  g[6] = f * (-0.5f * alpha * alpha) * fmaf(u, th, -lncosh);
  g[7] = f * alpha * u * th * iz0;
  g[8] = 0.f;
  g[9] = 0.f;
  return f;
}

__device__ __forceinline__ float ferrers_f(const CompF32 &c, float xp, float yp, float s) {
  const float yd = fmaf(s, c.s4, yp * c.s3);
  const float zd = fmaf(-s, c.s3, yp * c.s4);
  const float xb = fmaf(xp, c.s5, yd * c.s6);
  const float yb = fmaf(-xp, c.s6, yd * c.s5);
  const float m2 = fmaf(yb * yb, c.subScale, fmaf(xb * xb, c.subInner, zd * zd * c.subSmallK));
  if (!(m2 < 1.f)) return 0.f;
  return c.s0 * fast_ex2(c.s7 * fast_lg2(1.f - m2));
}

// value and d/d(X0, Y0, PA, inc, barPA, J_0, R_bar, q, q_z, n)
__device__ __forceinline__ float ferrers_fg(const CompF32 &c, float xp, float yp, float s, float *g) {
  const float ci = c.s3, si = c.s4, cb = c.s5, sb = c.s6;
  const float ia2 = c.subScale, ib2 = c.subInner, ic2 = c.subSmallK, n = c.s7;
  const float yd = fmaf(s, si, yp * ci);
  const float zd = fmaf(-s, ci, yp * si);
  const float xb = fmaf(xp, cb, yd * sb);
  const float yb = fmaf(-xp, sb, yd * cb);
  const float m2 = fmaf(yb * yb, ia2, fmaf(xb * xb, ib2, zd * zd * ic2));
  if (!(m2 < 1.f)) {
#pragma unroll
    for (int q = 0; q < kLosGrad; q++) g[q] = 0.f;
    return 0.f;
  }
  const float lW = fast_lg2(1.f - m2);
  const float P = fast_ex2(n * lW);
  const float f = c.s0 * P;
  const float fm = -n * c.s0 * fast_ex2((n - 1.f) * lW);  // df/dm^2
  const float dxb = 2.f * xb * ib2 * fm, dyb = 2.f * yb * ia2 * fm;
  const float fxp = fmaf(dxb, cb, -dyb * sb);
  const float fyd = fmaf(dxb, sb, dyb * cb);
  const float fzd = 2.f * zd * ic2 * fm;
  const float gp = fmaf(fyd, ci, fzd * si);
  g[0] = fmaf(-c.cosPA, fxp, c.sinPA * gp);
  g[1] = fmaf(-c.sinPA, fxp, -c.cosPA * gp);
  g[2] = kDeg2RadF * fmaf(fxp, yp, -gp * xp);
  g[3] = kDeg2RadF * fmaf(fyd, fmaf(s, ci, -yp * si), fzd * fmaf(yp, ci, s * si));
  g[4] = kDeg2RadF * 2.f * fm * xb * yb * (ib2 - ia2);
  g[5] = P;
  g[6] = fm * (-2.f * m2 * __fdividef(1.f, c.s1));
  g[7] = fm * (-2.f * xb * xb * ib2 * __fdividef(1.f, c.s2));
  g[8] = fm * (-2.f * zd * zd * ic2 * __fdividef(1.f, c.pad));
  g[9] = f * lW * kLn2F;
  return f;
}

__device__ __forceinline__ float los_f(const CompF32 &c, float xp, float yp, float s) {
  return c.type == F_EXPDISK3D ? expdisk_f(c, xp, yp, s) : ferrers_f(c, xp, yp, s);
}

// number of function parameters of a 3-D component
__device__ __forceinline__ int los_nparams(const CompF32 &c) { return c.type == F_EXPDISK3D ? 6 : 8; }

// ---------------------------------------------------------- warp rule
// The node (on [-1,1]) and Kronrod / Gauss weights this lane evaluates:
// lanes 0..9 the negative abscissae, 10..19 the positive ones, 20 the centre,
// 21..31 none.  Computed once per kernel (FP64 table -> FP32).
struct GkLane {
  float x, wk, wg;
};

__device__ __forceinline__ GkLane gk21_lane() {
  const int lane = threadIdx.x & 31;
  GkLane n{0.f, 0.f, 0.f};
  if (lane < 21) {
    const int k = lane < 10 ? lane : (lane < 20 ? lane - 10 : 10);
    const float xa = (float)GK21_XGK[k];
    n.x = lane < 10 ? -xa : xa;
    n.wk = (float)GK21_WGK[k];
    n.wg = (k & 1) ? (float)GK21_WG[k >> 1] : 0.f;
  }
  return n;
}

__device__ __forceinline__ void los_panel(const CompF32 &c, float xp, float yp, float lo, float hi,
                                          const GkLane &nd, float &res, float &err) {
  const float mid = 0.5f * (lo + hi), half = 0.5f * (hi - lo);
  const float f = (nd.wk != 0.f) ? los_f(c, xp, yp, fmaf(half, nd.x, mid)) : 0.f;
  const float K = los_wsum(nd.wk * f), G = los_wsum(nd.wg * f);
  res = K * half;
  err = fabsf((K - G) * half);
}

// Adaptive partition of the line of sight of one pixel (all lanes of the
// warp call it with the same arguments).  Lane p < np ends up holding panel
// p in [lo, hi]; returns np (0 when the integrand is zero everywhere) and the
// integral in 'total' (same in every lane).
__device__ __forceinline__ int los_partition(const CompF32 &c, float xp, float yp, const GkLane &nd,
                                             float &myLo, float &myHi, float &total) {
  const int lane = threadIdx.x & 31;
  float a, b, bp[2];
  int nbp = 0;
  if (c.type == F_EXPDISK3D) {
    b = c.subInner;
    a = -b;
    const float ci = c.s3, si = c.s4;
    if (si > 1e-6f) {
      const float t = -yp * ci / si;  // y_d = 0
      if (t > a && t < b) bp[nbp++] = t;
    }
    if (ci > 1e-6f) {
      const float t = yp * si / ci;  // z_d = 0
      if (t > a && t < b) bp[nbp++] = t;
    }
    if (nbp == 2) {
      if (bp[0] > bp[1]) {
        const float t = bp[0];
        bp[0] = bp[1];
        bp[1] = t;
      }
      if (!(bp[1] > bp[0])) nbp = 1;
    }
  } else {
    // chord of the ellipsoid: m^2(s) = A s^2 + 2 B s + C
    const float ci = c.s3, si = c.s4, cb = c.s5, sb = c.s6;
    const float ia2 = c.subScale, ib2 = c.subInner, ic2 = c.subSmallK;
    const float yd0 = yp * ci, zd0 = yp * si;
    const float xb0 = fmaf(xp, cb, yd0 * sb), xb1 = si * sb;
    const float yb0 = fmaf(-xp, sb, yd0 * cb), yb1 = si * cb;
    const float z1 = -ci;
    const float A = fmaf(yb1 * yb1, ia2, fmaf(xb1 * xb1, ib2, z1 * z1 * ic2));
    const float B = fmaf(yb0 * yb1, ia2, fmaf(xb0 * xb1, ib2, zd0 * z1 * ic2));
    const float C = fmaf(yb0 * yb0, ia2, fmaf(xb0 * xb0, ib2, zd0 * zd0 * ic2));
    const float D = fmaf(B, B, -A * (C - 1.f));
    if (!(A > 0.f) || !(D > 0.f)) {
      total = 0.f;
      return 0;
    }
    const float sq = sqrtf(D);
    const float qv = -(B + copysignf(sq, B));
    float s1 = qv / A, s2 = (qv != 0.f) ? (C - 1.f) / qv : -s1;
    if (s1 > s2) {
      const float t = s1;
      s1 = s2;
      s2 = t;
    }
    const float L = c.q;
    a = fmaxf(s1, -L);
    b = fminf(s2, L);
    if (!(b > a)) {
      total = 0.f;
      return 0;
    }
  }
  int np = 0;
  float myRes = 0.f, myErr = 0.f;
  myLo = 0.f;
  myHi = 0.f;
  float lo = a;
  for (int i = 0; i <= nbp; i++) {
    const float hi = (i < nbp) ? bp[i] : b;
    float r, e;
    los_panel(c, xp, yp, lo, hi, nd, r, e);
    if (lane == np) {
      myLo = lo;
      myHi = hi;
      myRes = r;
      myErr = e;
    }
    np++;
    lo = hi;
  }
  float tot;
  for (;;) {
    tot = los_wsum(lane < np ? myRes : 0.f);
    const float etot = los_wsum(lane < np ? myErr : 0.f);
    if (!(etot > kLosEpsRelFast * fabsf(tot)) || np >= kLosMaxPanels) break;
    float e = lane < np ? myErr : -1.f;
    int id = lane;
    for (int o = 16; o > 0; o >>= 1) {
      const float e2 = __shfl_xor_sync(0xffffffffu, e, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, id, o);
      if (e2 > e || (e2 == e && i2 < id)) {
        e = e2;
        id = i2;
      }
    }
    const float plo = __shfl_sync(0xffffffffu, myLo, id), phi = __shfl_sync(0xffffffffu, myHi, id);
    const float m = 0.5f * (plo + phi);
    if (!(m > plo && m < phi)) break;
    float r1, e1, r2, e2;
    los_panel(c, xp, yp, plo, m, nd, r1, e1);
    los_panel(c, xp, yp, m, phi, nd, r2, e2);
    if (lane == id) {
      myHi = m;
      myRes = r1;
      myErr = e1;
    }
    if (lane == np) {
      myLo = m;
      myHi = phi;
      myRes = r2;
      myErr = e2;
    }
    np++;
  }
  total = tot;
  return np;
}

// Value of a 3-D component at a pixel (xp, yp in its rotated frame).
__device__ __forceinline__ float los_value_warp(const CompF32 &c, float xp, float yp, const GkLane &nd) {
  float lo, hi, total;
  los_partition(c, xp, yp, nd, lo, hi, total);
  return total;
}

// d(value)/d(X0, Y0, function parameters) over the same panels; every lane
// returns the full sums in g[0..kLosGrad).
// Derivative integrals over a given partition (lane p < np holds panel p).
__device__ __forceinline__ void los_grad_panels(const CompF32 &c, float xp, float yp, const GkLane &nd, int np,
                                                float myLo, float myHi, float *g) {
  float acc[kLosGrad];
#pragma unroll
  for (int q = 0; q < kLosGrad; q++) acc[q] = 0.f;
  for (int p = 0; p < np; p++) {
    const float lo = __shfl_sync(0xffffffffu, myLo, p), hi = __shfl_sync(0xffffffffu, myHi, p);
    if (nd.wk != 0.f) {
      const float mid = 0.5f * (lo + hi), half = 0.5f * (hi - lo);
      const float s = fmaf(half, nd.x, mid);
      float t[kLosGrad];
      if (c.type == F_EXPDISK3D)
        expdisk_fg(c, xp, yp, s, t);
      else
        ferrers_fg(c, xp, yp, s, t);
      const float w = nd.wk * half;
#pragma unroll
      for (int q = 0; q < kLosGrad; q++) acc[q] = fmaf(w, t[q], acc[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < kLosGrad; q++) g[q] = los_wsum(acc[q]);
}

__device__ __forceinline__ void los_grad_warp(const CompF32 &c, float xp, float yp, const GkLane &nd, float *g) {
  float myLo, myHi, total;
  const int np = los_partition(c, xp, yp, nd, myLo, myHi, total);
  los_grad_panels(c, xp, yp, nd, np, myLo, myHi, g);
}

}  // namespace imfit
