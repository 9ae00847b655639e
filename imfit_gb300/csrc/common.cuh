// common.cuh -- shared types and per-component evaluators for the GB300
// model-image / fit-statistic kernels.
//
// Two evaluation forms exist for every image function:
//   * an FP64 form that restates the reference's FunctionObject::Setup /
//     GetValue arithmetic operation for operation (the "plain" drop-in path;
//     the translation unit that instantiates it is compiled with --fmad=false
//     so no a*b+c is contracted, as in the reference's x86 build);
//   * an FP32 form for the batched fast path: per-component geometry and the
//     Sersic b_n are prepared in FP64 once per parameter vector, pixel offsets
//     from component centres are formed exactly (integer part + FP64-rounded
//     fractional remainder), and the profile is evaluated with the SFU
//     (lg2/ex2) -- together with its analytic derivatives for the gradient.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace imfit {

enum FuncType : int {
  F_NONE = 0,
  F_SERSIC = 1,      // function_objects/func_sersic.cpp
  F_EXP = 2,         // function_objects/func_exp.cpp
  F_FLATSKY = 3,     // function_objects/func_flatsky.cpp
  F_GRING = 4,       // function_objects/func_gaussian-ring.cpp
  F_MOFFAT = 5,      // function_objects/func_moffat.cpp
  F_GAUSS = 6,       // function_objects/func_gaussian.cpp
  F_EXPDISK3D = 7,   // function_objects/func_expdisk3d.cpp
  F_FERRERS3D = 8,   // function_objects/func_ferrersbar3d.cpp
  F_POINTSOURCE = 9,     // function_objects/func_pointsource.cpp
  F_POINTSOURCEROT = 10, // function_objects/func_pointsource-rot.cpp
  F_TILTEDSKY = 11,      // function_objects/func_tilted-sky-plane.cpp
};

// 3-D classes: the value is a line-of-sight integral (func_expdisk3d.cpp,
// func_ferrersbar3d.cpp).
__host__ __device__ inline bool is_los(int t) { return t == F_EXPDISK3D || t == F_FERRERS3D; }

// PointSource classes are added after the convolution (IsPointSource,
// core/model_object.cpp:1163-1216), from an interpolated PSF.
__host__ __device__ inline bool is_point_source(int t) { return t == F_POINTSOURCE || t == F_POINTSOURCEROT; }

// classes without a position angle
__host__ __device__ inline bool has_pa(int t) {
  return t != F_FLATSKY && t != F_POINTSOURCE && t != F_TILTEDSKY;
}

constexpr int kMaxComponents = 32;
constexpr int kMaxParams = 256;
constexpr double kDeg2Rad = 0.017453292519943295;  // func_sersic.cpp:64
constexpr double kLog2e = 1.4426950408889634;
constexpr double kLn2 = 0.6931471805599453;

// Static description of one component (fixed for the lifetime of a model).
struct CompDesc {
  int type;
  int subsample;    // FunctionObject::SetSubsampling flag
  int paramOffset;  // first of this function's parameters in the parameter vector
  int x0Index;      // index of its function set's X0 (Y0 follows)
  int nParams;
  int background;   // 1 = spatially constant (FlatSky): added after convolution
  int psScale;      // point sources: PointSource::oversamplingScale on the main grid
  int pad1;
};

// FP64 Setup() state, restating each class's Setup (plain path).
struct CompF64 {
  int type, subsample, pad0, pad1;
  double x0, y0;
  double cosPA, sinPA, q;
  double a, b, c, d, e, f;      // type-specific (see comp_setup64)
  double g, h, i, j, k, l, m;   // 3-D functions
};

// FP32 fast-path state prepared once per parameter vector.
struct CompF32 {
  int type, subsample, paramOffset, x0Index;
  int x0i, y0i;        // integer parts of the centre
  float x0r, y0r;      // fractional remainders (FP64 difference rounded once)
  float cosPA, sinPA, invq, q;
  float s0, s1, s2, s3, s4, s5, s6, s7;  // type-specific, see comp_setup32
  float subScale;      // scale length used by the subsampling rule
  float subInner;      // inner radius of the constant 20x20 rule (4 Sersic, 3 others)
  float subSmallK;     // 20 (Sersic/Exp) or 40 (Moffat/Gaussian)
  float pad;
};

// ---------------------------------------------------------------------------
// Sersic b_n (function_objects/helper_funcs.cpp:14-29) and its derivative.
__host__ __device__ inline double sersic_bn(double n) {
  double n2 = n * n, b_n;
  if (n > 0.36) {
    b_n = 2 * n - 0.333333333333333 + 0.009876543209876543 / n + 0.0018028610621203215 / n2 +
          0.00011409410586365319 / (n2 * n) - 7.1510122958919723e-05 / (n2 * n2);
  } else {
    b_n = 0.01945 + -0.8902 * n + 10.95 * n2 + -19.67 * n2 * n + 13.43 * n2 * n2;
  }
  return b_n;
}

__host__ __device__ inline double sersic_dbn_dn(double n) {
  double n2 = n * n;
  if (n > 0.36) {
    return 2.0 - 0.009876543209876543 / n2 - 2.0 * 0.0018028610621203215 / (n2 * n) -
           3.0 * 0.00011409410586365319 / (n2 * n2) + 4.0 * 7.1510122958919723e-05 / (n2 * n2 * n);
  }
  return -0.8902 + 2.0 * 10.95 * n + 3.0 * -19.67 * n2 + 4.0 * 13.43 * n2 * n;
}

// ---------------------------------------------------------------------------
// FP64 Setup (plain path).  Field use per type:
//   Sersic:   a=n b=I_e c=r_e d=bn e=invn
//   Exp:      a=I_0 b=h
//   FlatSky:  a=I_sky
//   TiltedSkyPlane: a=I_0 b=m_x c=m_y
//   GRing:    a=A b=R_ring c=sigma_r d=2 sigma^2
//   Moffat:   a=I_0 b=fwhm c=beta d=alpha
//   Gaussian: a=I_0 b=sigma d=2 sigma^2
//   ExpDisk3D:    a=J_0 b=h c=n d=z_0 e=cosInc f=sinInc g=alpha h=scaledZ0 i=2^alpha
//   FerrersBar3D: a=J_0 b=R_bar e=cosInc f=sinInc g=cosBarPA h=sinBarPA i=a2 j=b2 k=c2 l=n m=limit
__host__ __device__ inline void comp_setup64(CompF64 &c, int type, int subsample, const double *p,
                                             double xc, double yc) {
  c.type = type;
  c.subsample = subsample;
  c.x0 = xc;
  c.y0 = yc;
  c.q = 1.0;
  c.cosPA = 1.0;
  c.sinPA = 0.0;
  if (has_pa(type)) {
    double par = (p[0] + 90.0) * kDeg2Rad;
    c.cosPA = cos(par);
    c.sinPA = sin(par);
  }
  switch (type) {
    case F_SERSIC:  // func_sersic.cpp:109-127
      c.q = 1.0 - p[1];
      c.a = p[2]; c.b = p[3]; c.c = p[4];
      c.d = sersic_bn(p[2]);
      c.e = 1.0 / p[2];
      break;
    case F_EXP:  // func_exp.cpp:104-119
      c.q = 1.0 - p[1];
      c.a = p[2]; c.b = p[3];
      break;
    case F_FLATSKY:  // func_flatsky.cpp:85-90
      c.a = p[0];
      break;
    case F_TILTEDSKY:  // func_tilted-sky-plane.cpp:85-93
      c.a = p[0]; c.b = p[1]; c.c = p[2];
      break;
    case F_POINTSOURCE:  // func_pointsource.cpp:206-211
      c.a = p[0];
      break;
    case F_POINTSOURCEROT:  // func_pointsource-rot.cpp:210-221 (PA + 90 as above)
      c.a = p[1];
      break;
    case F_GRING:  // func_gaussian-ring.cpp:102-121
      c.q = 1.0 - p[1];
      c.a = p[2]; c.b = p[3]; c.c = p[4];
      c.d = 2.0 * p[4] * p[4];
      break;
    case F_MOFFAT: {  // func_moffat.cpp:111-131
      c.q = 1.0 - p[1];
      c.a = p[2]; c.b = p[3]; c.c = p[4];
      double exponent = pow(2.0, 1.0 / p[4]);
      c.d = 0.5 * p[3] / sqrt(exponent - 1.0);
      break;
    }
    case F_GAUSS:  // func_gaussian.cpp:104-119
      c.q = 1.0 - p[1];
      c.a = p[2]; c.b = p[3];
      c.d = 2.0 * p[3] * p[3];
      break;
    case F_EXPDISK3D: {  // func_expdisk3d.cpp:149-171
      c.a = p[2]; c.b = p[3]; c.c = p[4]; c.d = p[5];
      c.e = cos(p[1] * kDeg2Rad);
      c.f = sin(p[1] * kDeg2Rad);
      c.g = 2.0 / p[4];
      c.h = c.g * p[5];
      c.i = pow(2.0, c.g);
      break;
    }
    case F_FERRERS3D: {  // func_ferrersbar3d.cpp:125-165
      c.a = p[3]; c.b = p[4];
      c.e = cos(p[1] * kDeg2Rad);
      c.f = sin(p[1] * kDeg2Rad);
      double bpa = (p[2] + 90.0) * kDeg2Rad;
      c.g = cos(bpa);
      c.h = sin(bpa);
      c.i = p[4] * p[4];
      c.j = p[5] * p[5] * c.i;
      c.k = p[6] * p[6] * c.i;
      c.l = p[7];
      double t = sqrt(c.j) * c.f;
      c.m = 1.01 * ((t < p[4]) ? p[4] : t);
      break;
    }
    default:
      break;
  }
}

// Number of subsamples per axis (CalculateSubsamples: func_sersic.cpp:197-213,
// func_exp.cpp:181-197, func_moffat.cpp:199-215, func_gaussian.cpp:182-198).
__host__ __device__ inline int n_subsamples64(const CompF64 &c, double r) {
  if (!c.subsample || !(r < 10.0)) return 1;
  double scale, rin;
  int small;
  switch (c.type) {
    case F_SERSIC: scale = c.c; rin = 4.0; small = 20; break;
    case F_EXP: scale = c.b; rin = 3.0; small = 20; break;
    case F_MOFFAT: scale = c.d; rin = 3.0; small = 40; break;
    case F_GAUSS: scale = c.b; rin = 3.0; small = 40; break;
    default: return 1;
  }
  int ns;
  if ((scale <= 1.0) && (r <= 1.0)) {
    int k = (int)(small / scale);
    ns = (k < 100) ? k : 100;
  } else if (r <= rin) {
    ns = 20;
  } else {
    int k = (int)(20 / r);
    ns = (k < 100) ? k : 100;
  }
  return ns;
}

// CalculateIntensity(r) of the radial classes, FP64.
__host__ __device__ inline double radial64(const CompF64 &c, double r) {
  switch (c.type) {
    case F_SERSIC: return c.b * exp(-c.d * (pow((r / c.c), c.e) - 1.0));
    case F_EXP: return c.a * exp(-r / c.b);
    case F_GRING: {
      double rd = fabs(r - c.b);
      return c.a * exp(-(rd * rd) / c.d);
    }
    case F_MOFFAT: {
      double sr = r / c.d;
      return c.a / pow((1.0 + sr * sr), c.c);
    }
    case F_GAUSS: {
      double r2 = r * r;
      return c.a * exp(-r2 / c.d);
    }
    default: return 0.0;
  }
}

// GetValue(x,y) for the 2-D classes, FP64, reference expression order
// (func_sersic.cpp:147-189; identical structure in the other radial classes).
__host__ __device__ inline double comp_value64_2d(const CompF64 &c, double x, double y) {
  if (c.type == F_FLATSKY) return c.a;
  if (c.type == F_TILTEDSKY) return c.a + c.b * (x - c.x0) + c.c * (y - c.y0);  // func_tilted-sky-plane.cpp:98-104
  double x_diff = x - c.x0, y_diff = y - c.y0;
  double xp = x_diff * c.cosPA + y_diff * c.sinPA;
  double yps = (-x_diff * c.sinPA + y_diff * c.cosPA) / c.q;
  double r = sqrt(xp * xp + yps * yps);
  int ns = n_subsamples64(c, r);
  if (ns > 1) {
    double d = 1.0 / ns;
    double xs0 = x - 0.5 + 0.5 * d;
    double ys0 = y - 0.5 + 0.5 * d;
    double sum = 0.0;
    for (int ii = 0; ii < ns; ii++) {
      double xi = xs0 + ii * d;
      for (int jj = 0; jj < ns; jj++) {
        double yi = ys0 + jj * d;
        x_diff = xi - c.x0;
        y_diff = yi - c.y0;
        xp = x_diff * c.cosPA + y_diff * c.sinPA;
        yps = (-x_diff * c.sinPA + y_diff * c.cosPA) / c.q;
        r = sqrt(xp * xp + yps * yps);
        sum += radial64(c, r);
      }
    }
    return sum / (ns * ns);
  }
  return radial64(c, r);
}

// ---------------------------------------------------------------------------
// FP32 fast form.
//
// Type-specific fields of CompF32 (all derived in FP64, rounded once):
//   Sersic:   s0=I_e s1=B=bn*log2(e) s2=log2(r_e) s3=1/n s4=bn s5=dbn/dn s6=n s7=r_e pad=1/r_e
//   Exp:      s0=I_0 s1=log2(e)/h s2=h s3=1/h
//   GRing:    s0=A s1=R s2=log2(e)/(2 sigma^2) s3=sigma s4=1/sigma^2 pad=1/sigma
//   Moffat:   s0=I_0 s1=1/alpha^2 s2=beta s3=alpha s4=fwhm s5=d(alpha)/d(beta) s6=1/alpha s7=1/fwhm
//   Gaussian: s0=I_0 s1=log2(e)/(2 sigma^2) s2=sigma s3=1/sigma s4=1/sigma^2
// (reciprocals are formed in FP64 at setup so the pixel loops divide nowhere)
//   FlatSky:  s0=I_sky
//   TiltedSkyPlane: s0=I_0 s1=m_x s2=m_y
//   ExpDisk3D:    s0=J_0 s1=1/h s2=h s3=cos(inc) s4=sin(inc) s5=alpha=2/n
//                 s6=1/(alpha z_0) s7=z_0 subScale=n subInner=20h (half-range)
//   FerrersBar3D: s0=J_0 s1=R_bar s2=q s3=cos(inc) s4=sin(inc) s5,s6=cos,sin(barPA+90)
//                 s7=n subScale=1/a^2 subInner=1/b^2 subSmallK=1/c^2 pad=q_z q=half-range
// The "E" factor below is the profile divided by its amplitude, so the
// amplitude derivative is E itself and zero amplitudes need no special case.

// FP64 transcendentals of a component's Setup, computed by separate warps
// (FP64 is a narrow pipe on this GPU: one long serial chain per component
// would dominate the set-up time).
struct SetupFP64 {
  double cosPA, sinPA;  // orientation (PA + 90 deg)
  double bn, dbn;       // Sersic b_n and db_n/dn
  double log2re;        // Sersic log2(r_e)
  double t;             // Moffat 2^(1/beta)
  // reciprocals, each computed by its own warp before the record is assembled
  double invq;          // 1 / (1 - ell)
  double inv3, inv4;    // 1 / p[3], 1 / p[4] (the types that divide by them)
  double invn;          // Sersic 1 / n
};

// Which reciprocals of SetupFP64 a type uses (setup work split over warps).
__host__ __device__ inline bool uses_invq(int t) {
  return t == F_SERSIC || t == F_EXP || t == F_GRING || t == F_MOFFAT || t == F_GAUSS;
}
__host__ __device__ inline bool uses_inv3(int t) { return t == F_EXP || t == F_MOFFAT || t == F_GAUSS; }
__host__ __device__ inline bool uses_inv4(int t) { return t == F_SERSIC || t == F_GRING; }

// b_n written in powers of 1/n (one division), same coefficients as
// function_objects/helper_funcs.cpp:14-29
__device__ inline void sersic_bn_horner(double n, double &bn, double &dbn) {
  if (n > 0.36) {
    const double v = 1.0 / n;
    const double c1 = 0.009876543209876543, c2 = 0.0018028610621203215;
    const double c3 = 0.00011409410586365319, c4 = -7.1510122958919723e-05;
    bn = 2.0 * n - 0.333333333333333 + v * (c1 + v * (c2 + v * (c3 + v * c4)));
    dbn = 2.0 - v * v * (c1 + v * (2.0 * c2 + v * (3.0 * c3 + v * 4.0 * c4)));
  } else {
    bn = sersic_bn(n);
    dbn = sersic_dbn_dn(n);
  }
}

__device__ inline void comp_setup32(CompF32 &o, const CompDesc &d, const double *params, const SetupFP64 &q) {
  const double *p = params + d.paramOffset;
  const double x0 = params[d.x0Index], y0 = params[d.x0Index + 1];
  o.type = d.type;
  o.subsample = d.subsample;
  o.paramOffset = d.paramOffset;
  o.x0Index = d.x0Index;
  const double xr = rint(x0), yr = rint(y0);
  o.x0i = (int)xr;
  o.y0i = (int)yr;
  o.x0r = (float)(x0 - xr);
  o.y0r = (float)(y0 - yr);
  o.cosPA = 1.f; o.sinPA = 0.f; o.q = 1.f; o.invq = 1.f;
  o.s0 = o.s1 = o.s2 = o.s3 = o.s4 = o.s5 = o.s6 = o.s7 = 0.f;
  o.subScale = 1.f; o.subInner = 3.f; o.subSmallK = 20.f;
  if (has_pa(d.type)) {
    o.cosPA = (float)q.cosPA;
    o.sinPA = (float)q.sinPA;
  }
  switch (d.type) {
    case F_SERSIC: {
      const double qq = 1.0 - p[1], n = p[2];
      o.q = (float)qq; o.invq = (float)q.invq;
      o.s0 = (float)p[3];
      o.s1 = (float)(q.bn * kLog2e);
      o.s2 = (float)q.log2re;
      o.s3 = (float)q.invn;
      o.s4 = (float)q.bn;
      o.s5 = (float)q.dbn;
      o.s6 = (float)n;
      o.s7 = (float)p[4];
      o.subScale = (float)p[4]; o.subInner = 4.f; o.subSmallK = 20.f;
      o.pad = (float)q.inv4;  // 1/r_e
      break;
    }
    case F_EXP: {
      const double qq = 1.0 - p[1];
      o.q = (float)qq; o.invq = (float)q.invq;
      o.s0 = (float)p[2];
      o.s1 = (float)(kLog2e * q.inv3);
      o.s2 = (float)p[3];
      o.s3 = (float)q.inv3;  // 1/h
      o.subScale = (float)p[3]; o.subInner = 3.f; o.subSmallK = 20.f;
      break;
    }
    case F_FLATSKY:
      o.s0 = (float)p[0];
      break;
    case F_TILTEDSKY:
      o.s0 = (float)p[0];
      o.s1 = (float)p[1];
      o.s2 = (float)p[2];
      break;
    case F_GRING: {
      const double qq = 1.0 - p[1], is2 = q.inv4 * q.inv4;
      o.q = (float)qq; o.invq = (float)q.invq;
      o.s0 = (float)p[2];
      o.s1 = (float)p[3];
      o.s2 = (float)(0.5 * kLog2e * is2);
      o.s3 = (float)p[4];
      o.s4 = (float)is2;       // 1/sigma^2
      o.pad = (float)q.inv4;   // 1/sigma
      break;
    }
    case F_MOFFAT: {
      const double qq = 1.0 - p[1];
      const double beta = p[4], fwhm = p[3], t = q.t;
      const double alpha = 0.5 * fwhm / sqrt(t - 1.0);
      o.q = (float)qq; o.invq = (float)q.invq;
      o.s0 = (float)p[2];
      o.s1 = (float)(1.0 / (alpha * alpha));
      o.s2 = (float)beta;
      o.s3 = (float)alpha;
      o.s4 = (float)fwhm;
      o.s5 = (float)(alpha * t * kLn2 / (2.0 * beta * beta * (t - 1.0)));
      o.s6 = (float)(1.0 / alpha);
      o.s7 = (float)q.inv3;  // 1/fwhm
      o.subScale = (float)alpha; o.subInner = 3.f; o.subSmallK = 40.f;
      break;
    }
    case F_GAUSS: {
      const double qq = 1.0 - p[1], is2 = q.inv3 * q.inv3;
      o.q = (float)qq; o.invq = (float)q.invq;
      o.s0 = (float)p[2];
      o.s1 = (float)(0.5 * kLog2e * is2);
      o.s2 = (float)p[3];
      o.s3 = (float)q.inv3;  // 1/sigma
      o.s4 = (float)is2;
      o.subScale = (float)p[3]; o.subInner = 3.f; o.subSmallK = 40.f;
      break;
    }
    case F_EXPDISK3D: {  // PA, inc, J_0, h, n, z_0 (func_expdisk3d.cpp:149-171)
      double si, ci;
      sincospi(p[1] / 180.0, &si, &ci);
      const double alpha = 2.0 / p[4];
      o.s0 = (float)p[2];                     // J_0
      o.s1 = (float)(1.0 / p[3]);             // 1/h
      o.s2 = (float)p[3];                     // h
      o.s3 = (float)ci;                       // cos(inc)
      o.s4 = (float)si;                       // sin(inc)
      o.s5 = (float)alpha;                    // 2/n
      o.s6 = (float)(1.0 / (alpha * p[5]));   // 1/(alpha z_0)
      o.s7 = (float)p[5];                     // z_0
      o.subScale = (float)p[4];               // n
      o.subInner = (float)(20.0 * p[3]);      // integration half-range 20 h
      break;
    }
    case F_FERRERS3D: {  // PA, inc, barPA, J_0, R_bar, q, q_z, n (func_ferrersbar3d.cpp:125-165)
      double si, ci, sb, cb;
      sincospi(p[1] / 180.0, &si, &ci);
      sincospi((p[2] + 90.0) / 180.0, &sb, &cb);
      const double a2 = p[4] * p[4], b2 = p[5] * p[5] * a2, c2 = p[6] * p[6] * a2;
      o.s0 = (float)p[3];                     // J_0
      o.s1 = (float)p[4];                     // R_bar
      o.s2 = (float)p[5];                     // q
      o.s3 = (float)ci;
      o.s4 = (float)si;
      o.s5 = (float)cb;                       // cos(barPA + 90)
      o.s6 = (float)sb;                       // sin(barPA + 90)
      o.s7 = (float)p[7];                     // n
      o.subScale = (float)(1.0 / a2);
      o.subInner = (float)(1.0 / b2);
      o.subSmallK = (float)(1.0 / c2);
      o.pad = (float)p[6];                    // q_z
      const double t = sqrt(b2) * si;
      o.q = (float)(1.01 * ((t < p[4]) ? p[4] : t));  // integration half-range
      break;
    }
    case F_POINTSOURCE:
      o.s0 = (float)p[0];  // I_tot
      o.s1 = (float)d.psScale;
      break;
    case F_POINTSOURCEROT:
      o.s0 = (float)p[1];  // I_tot
      o.s1 = (float)d.psScale;
      break;
    default:
      break;
  }
}

__device__ inline int n_subsamples32(const CompF32 &c, float r) {
  if (!c.subsample || !(r < 10.f)) return 1;
  if (c.type != F_SERSIC && c.type != F_EXP && c.type != F_MOFFAT && c.type != F_GAUSS) return 1;
  int ns;
  if (c.subScale <= 1.f && r <= 1.f) {
    int k = (int)(c.subSmallK / c.subScale);
    ns = k < 100 ? k : 100;
  } else if (r <= c.subInner) {
    ns = 20;
  } else {
    int k = (int)(20.f / r);
    ns = k < 100 ? k : 100;
  }
  return ns;
}

// Geometry of one (sub)pixel relative to a component centre.
struct Geo {
  float xp, yp, ys, r2;
};

__device__ inline Geo geo32(const CompF32 &c, float dx, float dy) {
  Geo g;
  g.xp = fmaf(dx, c.cosPA, dy * c.sinPA);
  g.yp = fmaf(-dx, c.sinPA, dy * c.cosPA);
  g.ys = g.yp * c.invq;
  g.r2 = fmaf(g.xp, g.xp, g.ys * g.ys);
  return g;
}

__device__ inline float fast_lg2(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ inline float fast_ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ inline float fast_sqrt(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Profile value of a radial component at squared radius r2 (FP32), for a
// component type fixed at compile time (the pixel loops are instantiated per
// type, so the per-pixel work carries no type dispatch and loads only the
// constants its type uses).
template <int TY>
__device__ __forceinline__ float radial_t(const CompF32 &c, float r2) {
  if constexpr (TY == F_SERSIC) {
    float lr = 0.5f * fast_lg2(r2);
    float u = fast_ex2((lr - c.s2) * c.s3);
    return c.s0 * fast_ex2(c.s1 - c.s1 * u);
  } else if constexpr (TY == F_EXP) {
    return c.s0 * fast_ex2(-fast_sqrt(r2) * c.s1);
  } else if constexpr (TY == F_GRING) {
    float d = fast_sqrt(r2) - c.s1;
    return c.s0 * fast_ex2(-d * d * c.s2);
  } else if constexpr (TY == F_MOFFAT) {
    return c.s0 * fast_ex2(-c.s2 * fast_lg2(fmaf(r2, c.s1, 1.f)));
  } else if constexpr (TY == F_GAUSS) {
    return c.s0 * fast_ex2(-r2 * c.s1);
  } else if constexpr (TY == F_FLATSKY) {
    return c.s0;
  } else {
    return 0.f;
  }
}

// The same with the type chosen at run time.
__device__ inline float radial32(const CompF32 &c, float r2) {
  switch (c.type) {
    case F_SERSIC: return radial_t<F_SERSIC>(c, r2);
    case F_EXP: return radial_t<F_EXP>(c, r2);
    case F_GRING: return radial_t<F_GRING>(c, r2);
    case F_MOFFAT: return radial_t<F_MOFFAT>(c, r2);
    case F_GAUSS: return radial_t<F_GAUSS>(c, r2);
    case F_FLATSKY: return radial_t<F_FLATSKY>(c, r2);
    default: return 0.f;
  }
}

// TiltedSkyPlane at offsets (dx, dy) from its function set's centre
// (func_tilted-sky-plane.cpp:98-104) and its derivatives, in the slot layout
// of radial_grad32 below: X0, Y0, I_0, m_x, m_y.  Returns 3.
__device__ inline float plane32(const CompF32 &c, float dx, float dy) { return fmaf(c.s1, dx, fmaf(c.s2, dy, c.s0)); }
__device__ inline int plane_grad32(const CompF32 &c, float dx, float dy, float scale, float *out) {
  out[0] = -scale * c.s1;
  out[1] = -scale * c.s2;
  out[2] = scale;
  out[3] = scale * dx;
  out[4] = scale * dy;
  return 3;
}

// Value of a component at pixel offset (dx,dy), with the reference's
// subsampling rule applied sequentially (used when a whole warp is not
// available, e.g. tiny tests).  nsOut receives the subsample count.
__device__ inline float comp_value32(const CompF32 &c, float dx, float dy, int *nsOut) {
  Geo g = geo32(c, dx, dy);
  int ns = n_subsamples32(c, fast_sqrt(g.r2));
  if (nsOut) *nsOut = ns;
  if (ns <= 1) return radial32(c, g.r2);
  float d = 1.f / ns, s = 0.f;
  float xs0 = dx - 0.5f + 0.5f * d, ys0 = dy - 0.5f + 0.5f * d;
  for (int ii = 0; ii < ns; ii++)
    for (int jj = 0; jj < ns; jj++) {
      Geo gs = geo32(c, xs0 + ii * d, ys0 + jj * d);
      s += radial32(c, gs.r2);
    }
  return s * (d * d);
}

// Function parameters of a radial type (the derivative slots after X0, Y0).
template <int TY>
__host__ __device__ constexpr int n_fparams() {
  return TY == F_SERSIC ? 5 : TY == F_EXP ? 4 : TY == F_GRING ? 5 : TY == F_MOFFAT ? 5 : TY == F_GAUSS ? 4
         : TY == F_TILTEDSKY ? 3 : 0;
}

// types whose GetValue subsamples near the centre (CalculateSubsamples)
template <int TY>
__host__ __device__ constexpr bool subsampling_t() {
  return TY == F_SERSIC || TY == F_EXP || TY == F_MOFFAT || TY == F_GAUSS;
}

// Analytic derivatives of one radial component at squared radius r2, for a
// type fixed at compile time:
// out[0..1] = d/dX0, d/dY0; out[2..] = d/d(function parameters in order), each
// multiplied by scale.  Returns the number of function parameters written
// after the two centre slots; *value (optional) receives the profile value.
template <int TY>
__device__ __forceinline__ int radial_grad_t(const CompF32 &c, const Geo &g, float scale, float *out,
                                             float *value = nullptr) {
  // 1/r from the SFU reciprocal square root, r = r2 / r (no IEEE division)
  const float rinv = (g.r2 > 0.f) ? rsqrtf(g.r2) : 0.f;
  const float r = g.r2 * rinv;
  float I, dIdr;
  constexpr int np = n_fparams<TY>();
  float pd[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // profile-parameter derivatives
  if constexpr (TY == F_SERSIC) {
    float lr = 0.5f * fast_lg2(g.r2);
    float u = fast_ex2((lr - c.s2) * c.s3);
    float E = fast_ex2(c.s1 - c.s1 * u);
    I = c.s0 * E;
    // dI/dr = -I bn u / (n r)
    float t = I * c.s4 * u * c.s3;
    dIdr = -t * rinv;
    // d/dn: -I [ bn'(u-1) - bn u ln(r/r_e) / n^2 ]
    float lnrr = (u > 0.f) ? (lr - c.s2) * (float)kLn2 : 0.f;
    pd[2] = -I * (c.s5 * (u - 1.f) - c.s4 * u * lnrr * c.s3 * c.s3);
    pd[3] = E;                 // d/dI_e
    pd[4] = t * c.pad;         // d/dr_e = I bn u / (n r_e)
  } else if constexpr (TY == F_EXP) {
    float E = fast_ex2(-r * c.s1);
    I = c.s0 * E;
    dIdr = -I * c.s3;
    pd[2] = E;                         // d/dI_0
    pd[3] = I * r * c.s3 * c.s3;       // d/dh
  } else if constexpr (TY == F_GRING) {
    float dd = r - c.s1;
    float E = fast_ex2(-dd * dd * c.s2);
    I = c.s0 * E;
    const float is2 = c.s4;
    dIdr = -I * dd * is2;
    pd[2] = E;                              // d/dA
    pd[3] = I * dd * is2;                   // d/dR_ring
    pd[4] = I * dd * dd * is2 * c.pad;      // d/dsigma_r
  } else if constexpr (TY == F_MOFFAT) {
    float D = fmaf(g.r2, c.s1, 1.f);
    float lD = fast_lg2(D);
    float E = fast_ex2(-c.s2 * lD);
    I = c.s0 * E;
    float Dinv = __fdividef(1.f, D);  // D >= 1
    dIdr = -2.f * I * c.s2 * r * c.s1 * Dinv;
    float dIdalpha = 2.f * I * c.s2 * g.r2 * c.s1 * Dinv * c.s6;
    pd[2] = E;                                             // d/dI_0
    pd[3] = dIdalpha * c.s3 * c.s7;                        // d/dfwhm
    pd[4] = -I * lD * (float)kLn2 + dIdalpha * c.s5;       // d/dbeta
  } else if constexpr (TY == F_GAUSS) {
    float E = fast_ex2(-g.r2 * c.s1);
    I = c.s0 * E;
    const float is2 = c.s4;
    dIdr = -I * r * is2;
    pd[2] = E;                              // d/dI_0
    pd[3] = I * g.r2 * is2 * c.s3;          // d/dsigma
  } else {
    return 0;
  }
  if (value) *value = I;
  // geometric chain rule; G = dI/dr / r
  const float G = dIdr * rinv;
  const float invq = c.invq;
  // dr/dX0 = (-xp cos + ys sin/q)/r ; dr/dY0 = (-xp sin - ys cos/q)/r
  out[0] = scale * G * (-g.xp * c.cosPA + g.ys * c.sinPA * invq);
  out[1] = scale * G * (-g.xp * c.sinPA - g.ys * c.cosPA * invq);
  // dr/dPA(deg) = deg2rad * xp * yp * (1 - 1/q^2) / r
  out[2] = scale * G * (float)kDeg2Rad * g.xp * g.yp * (1.f - invq * invq);
  // dr/dell = ys^2 / (q r)
  out[3] = scale * G * g.ys * g.ys * invq;
#pragma unroll
  for (int k = 2; k < 6; k++)
    if (k < np) out[2 + k] = scale * pd[k];
  return np;
}

// The same with the type chosen at run time.
__device__ inline int radial_grad32(const CompF32 &c, const Geo &g, float scale, float *out,
                                    float *value = nullptr) {
  switch (c.type) {
    case F_SERSIC: return radial_grad_t<F_SERSIC>(c, g, scale, out, value);
    case F_EXP: return radial_grad_t<F_EXP>(c, g, scale, out, value);
    case F_GRING: return radial_grad_t<F_GRING>(c, g, scale, out, value);
    case F_MOFFAT: return radial_grad_t<F_MOFFAT>(c, g, scale, out, value);
    case F_GAUSS: return radial_grad_t<F_GAUSS>(c, g, scale, out, value);
    default: return 0;
  }
}

}  // namespace imfit
