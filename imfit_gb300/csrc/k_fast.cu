// k_fast.cu -- batched FP32-evaluation / FP64-reduction path with the adjoint
// gradient.
//
// Per parameter vector b the statistic S(theta) and dS/dtheta are formed by
//   subsample  FP64 per-component geometry and Sersic b_n (FunctionObject::Setup)
//              by the first warps, then the subsampled box pixels of the main
//              window and of the oversampled region, warp-cooperatively,
//              into a table of values and derivatives
//   eval_r2c   model window rows evaluated in FP32 (SFU lg2/ex2), subsampled
//              pixels read from the table, then the row FFT -- the model
//              image never goes to HBM                         (CreateModelImage pixel loop)
//   cols       column FFT x PSF spectrum x inverse column FFT  (Convolver::ConvolveImage,
//              k_cols32.cu)
//   region     oversampled region: same pipeline at k x resolution and a
//              fused block-average that also forms the statistic terms and
//              adjoint seeds of the region's pixels, on a second stream
//              independent of the main window's until the final reduction
//                                                              (OversampledRegion, DownsampleAndReplace)
//   stat_rows  inverse row FFT, statistic terms in FP32 per pixel, summed in
//              double-float above the warp; the adjoint seed g = dS/dM
//              written and immediately row-FFT'd                (ChiSquared / CashStatistic)
//   cols(conj) the adjoint: correlation of g with the PSF
//   grad_rows  inverse row FFT, then one pass over the window accumulating
//              r~ * dm/dtheta for every parameter (table for subsampled
//              pixels), per-CTA double-float partials; the last CTA to finish
//              (a completion counter) forms the final sums in a fixed order.
// Consecutive kernels overlap their launch with the previous kernel's tail
// (programmatic dependent launch: each waits on griddepcontrol before reading
// what its predecessor wrote).
// The "valid" window W = N + P - 1 (rather than the reference's N + 2P model
// plus N + 3P - 1 padding) is exactly the set of model pixels the data
// crop depends on; constant backgrounds (FlatSky) are added after the
// convolution as I_sky * sum(PSF), which is what convolving a constant gives.
#include <algorithm>
#include <cstring>

#include "kernels.h"
#include "fft.cuh"
#include "ffsum.cuh"
#include "los_fast.cuh"

namespace imfit {

struct WinDesc {
  int cols, rows;
  int isRegion;
  int xOrig, yOrig;  // main: IRAF x = col + xOrig, y = row + yOrig
  int x1, y1, offX, offY, scale;
  float startOff, frac;
  float invScale;  // 1 / scale, correctly rounded
  int specPitch;
  long specBatch;
  cplx<float> *spec;
  // 3-D components: their summed line-of-sight values per window pixel
  // (forward) and the adjoint r~ per window pixel (gradient); null without them
  float *losVal, *losRt;
};

// floor(a / scale) for the window's scale: floor((a + 1/2) * (1/scale)) in
// FP32 with the correctly rounded reciprocal is exact for |a| < 2^21 and
// scales 1..128 (checked exhaustively), far beyond any window coordinate;
// four instructions instead of an integer division.
__device__ __forceinline__ int floordiv_scale(int a, float invScale) {
  return (int)floorf(((float)a + 0.5f) * invScale);
}

__device__ __forceinline__ bool subsampling_type(int t) {
  return t == F_SERSIC || t == F_EXP || t == F_MOFFAT || t == F_GAUSS;
}

// Offsets (dx, dy) of window pixel (row, col) from component c's centre,
// the integer parts exact and the fractions added once.  REG: the window is
// an oversampled region (fixed at compile time in the pixel loops, so the
// main window's loops carry none of the region's index arithmetic).
template <bool REG>
__device__ __forceinline__ void win_offsets_t(const WinDesc &w, const CompF32 &c, int row, int col, float &dx,
                                              float &dy) {
  int xi, yi;
  float xf = 0.f, yf = 0.f;
  if constexpr (!REG) {
    xi = col + w.xOrig;
    yi = row + w.yOrig;
  } else {
    const int tx = col + w.offX, ty = row + w.offY;
    const int qx = floordiv_scale(tx, w.invScale), qy = floordiv_scale(ty, w.invScale);
    xi = w.x1 + qx;
    yi = w.y1 + qy;
    xf = w.startOff + (float)(tx - qx * w.scale) * w.frac;
    yf = w.startOff + (float)(ty - qy * w.scale) * w.frac;
  }
  dx = (float)(xi - c.x0i) + (xf - c.x0r);
  dy = (float)(yi - c.y0i) + (yf - c.y0r);
}

__device__ __forceinline__ void win_offsets(const WinDesc &w, const CompF32 &c, int row, int col, float &dx,
                                            float &dy) {
  if (w.isRegion)
    win_offsets_t<true>(w, c, row, col, dx, dy);
  else
    win_offsets_t<false>(w, c, row, col, dx, dy);
}

// Rows [r0, r0 + n) meet component c's subsample box (rows [br0, br0 + side))?
// Only then can a pixel need the subsample table; the pixel loops of the
// other CTAs are compiled without the test.
__device__ __forceinline__ bool rows_meet_box(const CompF32 &c, int r0, int n, int br0, int side) {
  return c.subsample && subsampling_type(c.type) && r0 < br0 + side && br0 < r0 + n;
}

__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// pixel needs warp-cooperative subsampling for component c?
__device__ __forceinline__ int sub_count(const CompF32 &c, const Geo &g) {
  if (!c.subsample || !(g.r2 < 100.f)) return 1;
  return n_subsamples32(c, fast_sqrt(g.r2));
}

// --------------------------------------------------------------- setup
// FP64 Setup of component c of parameter vector b into rec (FunctionObject::
// Setup, core/model_object.cpp:1126-1135).  Each FP64 quantity -- the
// orientation (sincospi), Sersic b_n and log2 r_e, Moffat 2^(1/beta), the
// reciprocals the record needs, the background levels -- is computed by its
// own warp (FP64 operations have long latencies here: a transcendental takes
// about a microsecond), thread 0 then only assembles the FP32 record; all
// threads of the CTA call it.  With bg, also the constant background levels
// of vector b (FlatSky sum x sum of the PSF, main and region).
__device__ void setup_component(const FastArgs &a, int c, int b, CompF32 &rec, bool bg) {
  __shared__ SetupFP64 q;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const CompDesc d = a.desc[c];
  const double *P = a.params + (long)b * a.nParams;
  const double *p = P + d.paramOffset;
  if (lane == 0) {
    for (int task = w; task < 8; task += nw) {
      switch (task) {
        case 0:
          if (has_pa(d.type)) {
            double sn, cs;
            sincospi((p[0] + 90.0) * (1.0 / 180.0), &sn, &cs);
            q.cosPA = cs;
            q.sinPA = sn;
          }
          break;
        case 1:
          if (d.type == F_SERSIC) sersic_bn_horner(p[2], q.bn, q.dbn);
          if (d.type == F_MOFFAT) q.t = exp2(1.0 / p[4]);
          break;
        case 2:
          if (d.type == F_SERSIC) q.log2re = log2(p[4]);
          break;
        case 3:
          if (bg) {
            double s = 0.0;
            for (int k = 0; k < a.nComp; k++)
              if (a.desc[k].background) s += P[a.desc[k].paramOffset];
            a.bgLevel[2 * b] = (float)(s * a.psfSum);
            a.bgLevel[2 * b + 1] = (float)(s * a.psfSumOs);
          }
          break;
        case 4:
          if (uses_invq(d.type)) q.invq = 1.0 / (1.0 - p[1]);
          break;
        case 5:
          if (uses_inv3(d.type)) q.inv3 = 1.0 / p[3];
          break;
        case 6:
          if (uses_inv4(d.type)) q.inv4 = 1.0 / p[4];
          break;
        default:
          if (d.type == F_SERSIC) q.invn = 1.0 / p[2];
          break;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) comp_setup32(rec, d, P, q);
  __syncthreads();
}

// ------------------------------------------- subsampled pixels (precomputed)
// Offset of the table slot of (batch b, component c, window w).
__device__ __forceinline__ long sub_base(const FastArgs &a, int b, int c, int w) {
  const long areaM = (long)a.boxMain * a.boxMain, areaR = (long)a.boxReg * a.boxReg;
  return (((long)b * a.nComp + c) * (areaM + areaR) + (w ? areaM : 0)) * 8;
}

// components evaluated pixel by pixel in the row kernels (FlatSky and the
// point sources are added after the convolution, the 3-D classes by the
// line-of-sight kernels)
__device__ __forceinline__ bool in_rows(int t) { return t != F_FLATSKY && !is_los(t) && !is_point_source(t); }


// Box origin (window col, row) around a component centre.  Every pixel whose
// centre is within radius 10 of the component centre (the only ones the
// subsampling rule can touch) lies inside the box.
__device__ __forceinline__ void box_origin(const WinDesc &w, const CompF32 &c, int side, int &col0, int &row0) {
  if (!w.isRegion) {
    col0 = c.x0i - w.xOrig - (side / 2 - 1);
    row0 = c.y0i - w.yOrig - (side / 2 - 1);
  } else {
    const float tcx = ((float)(c.x0i - w.x1) + c.x0r - w.startOff) * (float)w.scale;
    const float tcy = ((float)(c.y0i - w.y1) + c.y0r - w.startOff) * (float)w.scale;
    col0 = (int)floorf(tcx) - w.offX - side / 2;
    row0 = (int)floorf(tcy) - w.offY - side / 2;
  }
}

// Lane's share of the ns x ns subsamples of one pixel: acc[0] += value,
// acc[1..] += derivatives (X0, Y0, then the function parameters).
template <int TY>
__device__ __forceinline__ void subsample_sum(const CompF32 &cc, int ns, float xs, float ys, float d, int lane,
                                              float *acc) {
  constexpr int NP = n_fparams<TY>();
  float o[7];
  const FastDiv byNs(ns);
  for (int t = lane; t < ns * ns; t += 32) {
    const int ii = byNs.div(t), jj = t - ii * ns;
    const Geo gs = geo32(cc, xs + ii * d, ys + jj * d);
    float v;
    radial_grad_t<TY>(cc, gs, 1.f, o, &v);
    acc[0] += v;
#pragma unroll
    for (int q = 0; q < 2 + NP; q++) acc[1 + q] += o[q];
  }
}

constexpr int kLatN = 20;  // subsample count of the shared lattice (see k_fast_region_lattice)

// Subsampled box pixels of one window.  The CTAs of (component, vector) take
// the box pixels round-robin (pixel p to CTA p mod gridDim), blockDim at a
// time: every thread classifies one pixel, the pixels that subsample go to
// two shared lists, and then
//   * pixels with at most kThreadNs^2 subsamples are summed by groups of
//     kGroup lanes (the lanes split the subsamples, a shuffle tree adds them);
//   * larger ones by a whole warp each -- lanes split the subsamples or, in
//     the oversampled region, pixels on the shared lattice sum their block of
//     it (lane i takes block column i).
// Table entry: [value, X0, Y0, function parameters...] averaged.
constexpr int kThreadNs = 5;
constexpr int kGroup = 8;

struct LatView {
  const float *lat;  // [8][U][U] of this (vector, component), or null
  int U, q0, q1, m;
};

template <int TY>
__device__ void subsample_pixels(const WinDesc &w, const CompF32 &cc, int side, int col0, int row0, float *tab,
                                 const LatView &L) {
  __shared__ int smallList[256], bigList[256];
  __shared__ int nSmall, nBig;
  constexpr int NP = n_fparams<TY>();
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5, warp = threadIdx.x >> 5;
  const FastDiv bySide(side);
  const int area = side * side;
  const int perCta = (area - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  auto offsets = [&](int p, int &pr, int &pc, float &dx, float &dy) {
    pr = bySide.div(p);
    pc = p - pr * side;
    const int row = row0 + pr, col = col0 + pc;
    if (row < 0 || row >= w.rows || col < 0 || col >= w.cols) return false;
    win_offsets(w, cc, row, col, dx, dy);
    return true;
  };
  for (int base = 0; base < perCta; base += blockDim.x) {
    if (threadIdx.x == 0) nSmall = nBig = 0;
    __syncthreads();
    const int i = base + (int)threadIdx.x;
    if (i < perCta) {
      const int p = (int)blockIdx.x + i * (int)gridDim.x;
      int pr, pc;
      float dx, dy;
      if (offsets(p, pr, pc, dx, dy)) {
        const int ns = sub_count(cc, geo32(cc, dx, dy));
        if (ns > kThreadNs)
          bigList[atomicAdd(&nBig, 1)] = p;
        else if (ns > 1)
          smallList[atomicAdd(&nSmall, 1)] = p;
      }
    }
    __syncthreads();
    // small counts: kGroup lanes per pixel, 32 / kGroup pixels per warp pass
    // (the loop bound is uniform over the warp: every lane reaches the shuffles)
    constexpr int kPer = 32 / kGroup;
    const int gl = lane % kGroup;
    for (int e0 = warp * kPer; e0 < nSmall; e0 += nw * kPer) {
      const int e = e0 + lane / kGroup;
      int ns = 0, p = 0;
      float dx = 0.f, dy = 0.f;
      if (e < nSmall) {
        int pr, pc;
        p = smallList[e];
        offsets(p, pr, pc, dx, dy);
        ns = sub_count(cc, geo32(cc, dx, dy));
      }
      const float d = ns > 0 ? 1.f / ns : 0.f, xs = dx - 0.5f + 0.5f * d, ys = dy - 0.5f + 0.5f * d;
      float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      float o[7];
      for (int t = gl; t < ns * ns; t += kGroup) {
        const int ii = t / ns, jj = t - ii * ns;
        const Geo gs = geo32(cc, xs + ii * d, ys + jj * d);
        float v;
        radial_grad_t<TY>(cc, gs, 1.f, o, &v);
        acc[0] += v;
#pragma unroll
        for (int q = 0; q < 2 + NP; q++) acc[1 + q] += o[q];
      }
#pragma unroll
      for (int q = 0; q < 8; q++)
#pragma unroll
        for (int off = kGroup / 2; off > 0; off >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], off);
      if (gl == 0 && ns > 0) {
        float *dst = tab + (long)p * 8;
#pragma unroll
        for (int q = 0; q < 8; q++) dst[q] = acc[q] * (d * d);
      }
    }
    // large counts: one warp per pixel
    for (int e = warp; e < nBig; e += nw) {
      const int p = bigList[e];
      int pr, pc;
      float dx, dy;
      offsets(p, pr, pc, dx, dy);
      const int ns = sub_count(cc, geo32(cc, dx, dy));
      const float d = 1.f / ns;
      float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (L.lat && ns == kLatN && pr >= L.q0 && pr <= L.q1 && pc >= L.q0 && pc <= L.q1) {
        if (lane < kLatN) {  // lane i: block column i (consecutive lanes read consecutive floats)
          const long ch = (long)L.U * L.U;
          const float *col = L.lat + (long)((pr - L.q0) * L.m) * L.U + (pc - L.q0) * L.m + lane;
#pragma unroll
          for (int q = 0; q < 8; q++) {
            float t = 0.f;
#pragma unroll
            for (int k = 0; k < kLatN; k++) t += col[q * ch + (long)k * L.U];
            acc[q] = t;
          }
        }
      } else {
        subsample_sum<TY>(cc, ns, dx - 0.5f + 0.5f * d, dy - 0.5f + 0.5f * d, d, lane, acc);
      }
#pragma unroll
      for (int q = 0; q < 8; q++) acc[q] = warp_sum(acc[q]);
      if (lane == 0) {
        float *dst = tab + (long)p * 8;
#pragma unroll
        for (int q = 0; q < 8; q++) dst[q] = acc[q] * (d * d);
      }
    }
    __syncthreads();
  }
}

// First kernel of an evaluation, on grid (x, c, b): every CTA sets up
// component c of parameter vector b in FP64 (each redundantly, so that no
// CTA waits for another), CTA x = 0 publishes the FP32 record, the subsample
// boxes of both windows and, for c = 0, the background levels and a zeroed
// completion counter for the final reduction; then the CTAs of a subsampling
// component fill the main window's subsample table, one warp per box pixel
// (grid-stride over the CTAs of (c, b)): the average over the pixel's ns x ns
// subsamples of the profile and of its 7 derivatives (X0, Y0, then the
// function parameters).
__global__ void __launch_bounds__(256) k_fast_setup_subsample(FastArgs a, WinDesc mw, WinDesc rw, int hasRegion) {
  pdl_wait();
  pdl_trigger();  // dependents still wait for this grid to complete
  const int b = blockIdx.z, c = blockIdx.y;
  __shared__ CompF32 rec;
  __shared__ int box[2];
  setup_component(a, c, b, rec, c == 0 && blockIdx.x == 0);
  const bool sub = rec.subsample && subsampling_type(rec.type);
  if (threadIdx.x == 0) {
    if (sub) box_origin(mw, rec, a.boxMain, box[0], box[1]);
    if (blockIdx.x == 0) {
      a.comps[b * a.nComp + c] = rec;
      if (c == 0 && a.done) a.done[b] = 0u;
      if (sub) {
        int *o = a.subBox + ((long)b * a.nComp + c) * 4;
        o[0] = box[0];
        o[1] = box[1];
        if (hasRegion) box_origin(rw, rec, a.boxReg, o[2], o[3]);
      }
    }
  }
  __syncthreads();
  if (!sub) return;
  const CompF32 cc = rec;
  float *tab = a.subTab + sub_base(a, b, c, 0);
  const LatView none{nullptr, 0, 0, 0, 0};
  switch (cc.type) {
    case F_SERSIC: subsample_pixels<F_SERSIC>(mw, cc, a.boxMain, box[0], box[1], tab, none); break;
    case F_EXP: subsample_pixels<F_EXP>(mw, cc, a.boxMain, box[0], box[1], tab, none); break;
    case F_MOFFAT: subsample_pixels<F_MOFFAT>(mw, cc, a.boxMain, box[0], box[1], tab, none); break;
    default: subsample_pixels<F_GAUSS>(mw, cc, a.boxMain, box[0], box[1], tab, none); break;
  }
}

// With an oversampled region the set-up and the main window's table are two
// kernels, so that the region's pipeline (side stream) can start after the
// set-up alone: CTA (c, b) sets up component c of parameter vector b in FP64
// and publishes what k_fast_setup_subsample's CTA x = 0 publishes.
__global__ void __launch_bounds__(256) k_fast_setup(FastArgs a, WinDesc mw, WinDesc rw, int hasRegion) {
  pdl_wait();
  pdl_trigger();  // dependents still wait for this grid to complete
  const int c = blockIdx.x, b = blockIdx.y;
  __shared__ CompF32 rec;
  setup_component(a, c, b, rec, c == 0);
  if (threadIdx.x == 0) {
    a.comps[b * a.nComp + c] = rec;
    if (c == 0 && a.done) a.done[b] = 0u;
    if (rec.subsample && subsampling_type(rec.type)) {
      int *o = a.subBox + ((long)b * a.nComp + c) * 4;
      box_origin(mw, rec, a.boxMain, o[0], o[1]);
      if (hasRegion) box_origin(rw, rec, a.boxReg, o[2], o[3]);
    }
  }
}

// Subsampled pixels of the main window: one warp per box pixel (grid-stride
// over the CTAs of component c, vector b), the average over the pixel's
// ns x ns subsamples of the profile and of its 7 derivatives (X0, Y0, then
// the function parameters).
__global__ void __launch_bounds__(256) k_fast_subsample(FastArgs a, WinDesc w) {
  pdl_wait();
  pdl_trigger();  // dependents still wait for this grid to complete
  const int b = blockIdx.z, c = blockIdx.y;
  const CompF32 cc = a.comps[b * a.nComp + c];
  if (!cc.subsample || !subsampling_type(cc.type)) return;
  const int *o = a.subBox + ((long)b * a.nComp + c) * 4;
  float *tab = a.subTab + sub_base(a, b, c, 0);
  const LatView none{nullptr, 0, 0, 0, 0};
  switch (cc.type) {
    case F_SERSIC: subsample_pixels<F_SERSIC>(w, cc, a.boxMain, o[0], o[1], tab, none); break;
    case F_EXP: subsample_pixels<F_EXP>(w, cc, a.boxMain, o[0], o[1], tab, none); break;
    case F_MOFFAT: subsample_pixels<F_MOFFAT>(w, cc, a.boxMain, o[0], o[1], tab, none); break;
    default: subsample_pixels<F_GAUSS>(w, cc, a.boxMain, o[0], o[1], tab, none); break;
  }
}

// ------------------------------- oversampled region: shared subsample lattice
// In an oversampled region (scale k) the subsamples of a pixel span a whole
// main-image pixel around its centre (the function's own GetValue, e.g.
// func_sersic.cpp:163-183, called at the subpixel centres), so neighbouring
// subpixels' subsample grids overlap.  The pixels within the constant-count
// radius have kLatN x kLatN subsamples; when k divides kLatN they all lie on
// one lattice of spacing 1 / kLatN, pixel (br, bc) covering the kLatN x kLatN
// block that starts at ((br - q0) m, (bc - q0) m), m = kLatN / k.  The
// lattice over the box pixels [q0, q0 + 2h] (h = a.latHalf, which covers
// radius 4 around the centre; q0 = side / 2 - h) is evaluated once, one
// thread per point (k_fast_region_lattice), and those pixels' table entries
// are its block sums (k_fast_region_sub, lane i summing block column i).  For
// the 1024x1024 benchmark model with its 40x40 region at k = 5: 2 x 188^2
// lattice points plus about 78,000 direct subsamples instead of 714,000
// direct subsamples.

template <int TY>
__device__ __forceinline__ void lattice_point(const CompF32 &cc, float x, float y, float *dst, long chStride) {
  constexpr int C = 3 + n_fparams<TY>();
  const Geo gs = geo32(cc, x, y);
  float o[7], v;
  radial_grad_t<TY>(cc, gs, 1.f, o, &v);
  dst[0] = v;
#pragma unroll
  for (int q = 0; q < C - 1; q++) dst[(q + 1) * chStride] = o[q];
#pragma unroll
  for (int q = C; q < 8; q++) dst[q * chStride] = 0.f;
}

__global__ void __launch_bounds__(256) k_fast_region_lattice(FastArgs a, WinDesc w) {
  pdl_wait();
  pdl_trigger();  // dependents still wait for this grid to complete
  const int b = blockIdx.z, c = blockIdx.y;
  const CompF32 cc = a.comps[b * a.nComp + c];
  if (!cc.subsample || !subsampling_type(cc.type)) return;
  const int U = a.latSide, side = a.boxReg, q0 = side / 2 - a.latHalf;
  const int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= U * U) return;
  const int yb = pt / U, xa = pt - yb * U;
  const int *o = a.subBox + ((long)b * a.nComp + c) * 4;
  float dx0, dy0;
  win_offsets(w, cc, o[3] + q0, o[2] + q0, dx0, dy0);
  const float d = 1.f / kLatN;
  const float x = dx0 - 0.5f + 0.5f * d + (float)xa * d, y = dy0 - 0.5f + 0.5f * d + (float)yb * d;
  const long chStride = (long)U * U;
  float *dst = a.lat + ((long)b * a.nComp + c) * 8 * chStride + pt;
  switch (cc.type) {
    case F_SERSIC: lattice_point<F_SERSIC>(cc, x, y, dst, chStride); break;
    case F_EXP: lattice_point<F_EXP>(cc, x, y, dst, chStride); break;
    case F_MOFFAT: lattice_point<F_MOFFAT>(cc, x, y, dst, chStride); break;
    default: lattice_point<F_GAUSS>(cc, x, y, dst, chStride); break;
  }
}

// Subsampled pixels of the oversampled region (subsample_pixels, with the
// shared lattice when there is one).
__global__ void __launch_bounds__(256) k_fast_region_sub(FastArgs a, WinDesc w) {
  pdl_wait();
  pdl_trigger();  // dependents still wait for this grid to complete
  const int b = blockIdx.z, c = blockIdx.y;
  const CompF32 cc = a.comps[b * a.nComp + c];
  if (!cc.subsample || !subsampling_type(cc.type)) return;
  const int side = a.boxReg;
  const int *o = a.subBox + ((long)b * a.nComp + c) * 4;
  float *tab = a.subTab + sub_base(a, b, c, 1);
  LatView L{nullptr, a.latSide, side / 2 - a.latHalf, side / 2 + a.latHalf, kLatN / w.scale};
  if (a.lat) L.lat = a.lat + ((long)b * a.nComp + c) * 8 * (long)a.latSide * a.latSide;
  switch (cc.type) {
    case F_SERSIC: subsample_pixels<F_SERSIC>(w, cc, side, o[2], o[3], tab, L); break;
    case F_EXP: subsample_pixels<F_EXP>(w, cc, side, o[2], o[3], tab, L); break;
    case F_MOFFAT: subsample_pixels<F_MOFFAT>(w, cc, side, o[2], o[3], tab, L); break;
    default: subsample_pixels<F_GAUSS>(w, cc, side, o[2], o[3], tab, L); break;
  }
}

// Subsampled value of component c at window pixel (row, col): table lookup,
// or (outside the box, which the radius bound rules out) a direct sum.
__device__ __forceinline__ float sub_value(const FastArgs &a, const int *box, int b, int c, int win,
                                           const CompF32 &cc, int row, int col, float dx, float dy) {
  const int side = win ? a.boxReg : a.boxMain;
  const int br = row - box[1], bc = col - box[0];
  if (br >= 0 && br < side && bc >= 0 && bc < side) return a.subTab[sub_base(a, b, c, win) + ((long)br * side + bc) * 8];
  return comp_value32(cc, dx, dy, nullptr);
}

// ------------------------------------------------------ eval + row r2c
// Adds component cc's value at every pixel of the CTA's rows to the row
// buffer (one thread per complex point = two pixels; every pass maps the
// same points to the same thread, so the passes need no barrier).
template <int TY, bool REG, bool BOX>
__device__ __forceinline__ void eval_pixels(const CompF32 cc, const WinDesc &w, int row0, int nl, int M, int ls,
                                            const FastDiv &byM, cplx<float> *buf, const float *tab, int side,
                                            int bc0, int br0) {
  for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
    const int l = byM.div(idx), k = idx - l * M;
    const int row = row0 + l;
    float v[2] = {0.f, 0.f};
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const int col = 2 * k + e;
      if (col >= w.cols) continue;
      float dx, dy;
      win_offsets_t<REG>(w, cc, row, col, dx, dy);
      if constexpr (TY == F_TILTEDSKY) {
        v[e] = plane32(cc, dx, dy);
      } else {
        const Geo g = geo32(cc, dx, dy);
        if (BOX && subsampling_t<TY>() && g.r2 < 100.f && n_subsamples32(cc, fast_sqrt(g.r2)) > 1) {
          // subsampled pixel: the precomputed table (a direct average outside
          // the box, which the radius bound rules out)
          const int br = row - br0, bc = col - bc0;
          v[e] = (br >= 0 && br < side && bc >= 0 && bc < side) ? tab[((long)br * side + bc) * 8]
                                                                : comp_value32(cc, dx, dy, nullptr);
        } else {
          v[e] = radial_t<TY>(cc, g.r2);
        }
      }
    }
    cplx<float> &z = buf[l * ls + k];
    z.x += v[0];
    z.y += v[1];
  }
}

// eval_pixels with the window kind and the box test chosen at run time
template <int TY>
__device__ __forceinline__ void eval_pixels_rt(bool reg, bool box, const CompF32 &cc, const WinDesc &w, int row0,
                                               int nl, int M, int ls, const FastDiv &byM, cplx<float> *buf,
                                               const float *tab, int side, int bc0, int br0) {
  if (reg) {
    if (box) eval_pixels<TY, true, true>(cc, w, row0, nl, M, ls, byM, buf, tab, side, bc0, br0);
    else eval_pixels<TY, true, false>(cc, w, row0, nl, M, ls, byM, buf, tab, side, bc0, br0);
  } else {
    if (box) eval_pixels<TY, false, true>(cc, w, row0, nl, M, ls, byM, buf, tab, side, bc0, br0);
    else eval_pixels<TY, false, false>(cc, w, row0, nl, M, ls, byM, buf, tab, side, bc0, br0);
  }
}

__global__ void __launch_bounds__(1024) k_fast_eval_r2c(FastArgs a, WinDesc w, FFTPlan<float> plan,
                                                       const cplx<float> *__restrict__ twL, int rpb, int win) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y;
  const int M = plan.n, ls = M + 1;
  CompF32 *sc = reinterpret_cast<CompF32 *>(smem);
  int *boxes = reinterpret_cast<int *>(sc + kMaxComponents);
  cplx<float> *bufA = reinterpret_cast<cplx<float> *>(boxes + 2 * kMaxComponents);
  cplx<float> *bufB = bufA + rpb * ls;
  const int nC = a.nComp;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) {
    sc[i] = a.comps[b * nC + i];
    const int *o = a.subBox + (((long)b * nC + i) * 2 + win) * 2;
    boxes[2 * i] = o[0];
    boxes[2 * i + 1] = o[1];
  }
  const int row0 = blockIdx.x * rpb;
  const int nl = min(rpb, w.rows - row0);
  __syncthreads();
  if (nl <= 0) return;
  const FastDiv byM(M), byM1(M + 1);
  for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
    const int l = byM.div(idx);
    bufA[l * ls + idx - l * M] = {0.f, 0.f};
  }
  const int side = win ? a.boxReg : a.boxMain;
  for (int c = 0; c < nC; c++) {
    const CompF32 cc = sc[c];
    if (!in_rows(cc.type)) continue;
    const float *tab = a.subTab + sub_base(a, b, c, win);
    const int bc0 = boxes[2 * c], br0 = boxes[2 * c + 1];
    const bool box = rows_meet_box(cc, row0, nl, br0, side);
    switch (cc.type) {
      case F_SERSIC: eval_pixels_rt<F_SERSIC>(w.isRegion, box, cc, w, row0, nl, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_EXP: eval_pixels_rt<F_EXP>(w.isRegion, box, cc, w, row0, nl, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_GRING: eval_pixels_rt<F_GRING>(w.isRegion, box, cc, w, row0, nl, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_MOFFAT: eval_pixels_rt<F_MOFFAT>(w.isRegion, box, cc, w, row0, nl, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_GAUSS: eval_pixels_rt<F_GAUSS>(w.isRegion, box, cc, w, row0, nl, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_TILTEDSKY: eval_pixels_rt<F_TILTEDSKY>(w.isRegion, box, cc, w, row0, nl, M, ls, byM, bufA, tab, side, bc0, br0); break;
      default: break;
    }
  }
  if (w.losVal) {  // the 3-D components' line-of-sight sums
    for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
      const int l = byM.div(idx), k = idx - l * M;
      const float *lv = w.losVal + ((long)b * w.rows + row0 + l) * w.cols;
      cplx<float> &z = bufA[l * ls + k];
      if (2 * k < w.cols) z.x += lv[2 * k];
      if (2 * k + 1 < w.cols) z.y += lv[2 * k + 1];
    }
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, plan, nl, ls, 1, -1, false);
  pdl_trigger();
  cplx<float> *out = w.spec + (long)b * w.specBatch;
  for (int idx = threadIdx.x; idx < nl * (M + 1); idx += blockDim.x) {
    const int l = byM1.div(idx), k = idx - l * (M + 1);
    out[(long)(row0 + l) * w.specPitch + k] = r2c_post(Z + l * ls, k, M, twL);
  }
}

// ------------------------------------------------------------ point sources
// Point source c at scaled offsets (xd, yd) = s (x - x0, y - y0) from its
// centre: the value I_tot P(xd, yd) (rotated by PA for PointSourceRot) and,
// when dv is given, its derivatives w.r.t. X0, Y0, I_tot and PA
// (func_pointsource.cpp:220-229, func_pointsource-rot.cpp:229-243).
__device__ __forceinline__ float ps_eval(const CompF32 &c, const PsfInterp<float> &ip, float xd, float yd, float s,
                                         float *dv) {
  float xa = xd, ya = yd;
  if (c.type == F_POINTSOURCEROT) {
    xa = xd * c.cosPA + yd * c.sinPA;
    ya = -xd * c.sinPA + yd * c.cosPA;
  }
  float P, Px, Py;
  psf_interp32(ip, xa, ya, P, Px, Py);
  const float I = c.s0;
  if (dv) {
    if (c.type == F_POINTSOURCEROT) {
      dv[0] = I * s * (-Px * c.cosPA + Py * c.sinPA);
      dv[1] = I * s * (-Px * c.sinPA - Py * c.cosPA);
      dv[3] = I * (Px * ya - Py * xa) * 0.017453292f;  // d theta / d PA = pi/180
    } else {
      dv[0] = -I * s * Px;
      dv[1] = -I * s * Py;
      dv[3] = 0.f;
    }
    dv[2] = P;
  }
  return I * P;
}

// the point source touches nothing beyond the PSF's half-diagonal
__device__ __forceinline__ bool ps_far(const PsfInterp<float> &ip, float xd, float yd) {
  return xd * xd + yd * yd > ip.xb * ip.xb + ip.yb * ip.yb;
}

// data pixel (row, col): offsets from point source c, unscaled
__device__ __forceinline__ void ps_offsets(const CompF32 &c, int row, int col, float &X, float &Y) {
  X = (float)(col + 1 - c.x0i) - c.x0r;
  Y = (float)(row + 1 - c.y0i) - c.y0r;
}

// Main grid: sum over the point sources at data pixel (row, col), each at its
// own current scale (CompF32::s1); with acc, also adds g * derivatives.
__device__ float ps_main(const FastArgs &a, int b, int row, int col, float g, float *acc) {
  float v = 0.f;
  for (int p = 0; p < a.nPs; p++) {
    const CompF32 &c = a.comps[b * a.nComp + a.psComp[p]];
    float X, Y;
    ps_offsets(c, row, col, X, Y);
    const float s = c.s1, xd = s * X, yd = s * Y;
    if (ps_far(a.psMain, xd, yd)) continue;
    float dv[4];
    v += ps_eval(c, a.psMain, xd, yd, s, acc ? dv : nullptr);
    if (acc)
      for (int q = 0; q < 4; q++) atomicAdd(acc + 4 * p + q, g * dv[q]);
  }
  return v;
}

// Oversampled region: sum over the k x k subpixels of data pixel (row, col)
// and over the point sources, at the region's scale with the region's
// interpolator (oversampled_region.cpp:363-408: subpixel x = x1 + (0.5/k - 0.5)
// + j/k, so k (x - x0) = k X - (k - 1)/2 + v); with acc, adds g * derivatives
// (dv: their subpixel sums).
__device__ float ps_region(const FastArgs &a, int k, int b, int row, int col, float g, float *acc) {
  float v = 0.f;
  const float s = (float)k, h = 0.5f * (float)(k - 1);
  for (int p = 0; p < a.nPs; p++) {
    const CompF32 &c = a.comps[b * a.nComp + a.psComp[p]];
    float X, Y;
    ps_offsets(c, row, col, X, Y);
    const float bx = s * X - h, by = s * Y - h;  // offsets of the first subpixel
    // nearest subpixel offsets to the centre along each axis
    const float nx = bx > 0.f ? bx : (bx + (float)(k - 1) < 0.f ? -(bx + (float)(k - 1)) : 0.f);
    const float ny = by > 0.f ? by : (by + (float)(k - 1) < 0.f ? -(by + (float)(k - 1)) : 0.f);
    if (ps_far(a.psReg, nx, ny)) continue;
    float sum[4] = {0.f, 0.f, 0.f, 0.f};
    for (int u = 0; u < k; u++)
      for (int w = 0; w < k; w++) {
        float dv[4];
        v += ps_eval(c, a.psReg, bx + (float)w, by + (float)u, s, acc ? dv : nullptr);
        if (acc)
          for (int q = 0; q < 4; q++) sum[q] += dv[q];
      }
    if (acc)
      for (int q = 0; q < 4; q++) atomicAdd(acc + 4 * p + q, g * sum[q]);
  }
  return v;
}

// ------------------------------------------------------------- reduce
// Double-float sums of the per-CTA partials of parameter vector b in a fixed
// order (deterministic), one warp per output quantity: the statistic, the
// background term and, with nGradBlocks > 0, every gradient entry.  Run by
// the last CTA of the evaluation's final pass (finish_cta), whose partials
// are then all written.
// Double-float sum of p[lane], p[lane + 32], ... below n: four independent
// loads in flight per lane, four partial sums combined in a fixed order.
__device__ __forceinline__ ffloat lane_sum(const float2 *p, int n, int lane) {
  ffloat t0 = {0.f, 0.f}, t1 = t0, t2 = t0, t3 = t0;
  int i = lane;
  for (; i + 96 < n; i += 128) {
    const float2 v0 = __ldcg(p + i), v1 = __ldcg(p + i + 32), v2 = __ldcg(p + i + 64), v3 = __ldcg(p + i + 96);
    t0 = ff_add(t0, ff_load(v0));
    t1 = ff_add(t1, ff_load(v1));
    t2 = ff_add(t2, ff_load(v2));
    t3 = ff_add(t3, ff_load(v3));
  }
  for (; i < n; i += 32) t0 = ff_add(t0, ff_load(__ldcg(p + i)));
  return ff_add(ff_add(t0, t1), ff_add(t2, t3));
}

__device__ void reduce_entry(const FastArgs &a, int b, int nGradBlocks) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int nq = 2 + (nGradBlocks > 0 ? a.nParams : 0);
  for (int j = wid; j < nq; j += nw) {
    ffloat t;
    if (j < 2) {
      t = lane_sum(a.statPart + ((long)b * 2 + j) * a.partStride, a.nStatBlocks, lane);
    } else {
      t = lane_sum(a.gradPart + ((long)b * a.nParams + (j - 2)) * a.partStride, nGradBlocks, lane);
      // point sources: partials of the statistic CTAs for the parameters they touch
      for (int ps = 0; ps < a.nPs; ps++) {
        const CompDesc &d = a.desc[a.psComp[ps]];
        const bool rot = d.type == F_POINTSOURCEROT;
        const int map[4] = {d.x0Index, d.x0Index + 1, d.paramOffset + (rot ? 1 : 0), rot ? d.paramOffset : -1};
        for (int q = 0; q < 4; q++) {
          if (map[q] != j - 2) continue;
          t = ff_add(t, lane_sum(a.psPart + ((long)b * 4 * a.nPs + 4 * ps + q) * a.partStride, a.nStatBlocks, lane));
        }
      }
    }
    t = ff_warp_sum(t);
    if (lane != 0) continue;
    const double v = ff_value(t);
    if (j == 0) {
      a.stat[b] = v;
    } else if (j == 1) {
      if (nGradBlocks > 0)
        for (int c = 0; c < a.nComp; c++)
          if (a.desc[c].background) a.grad[(long)b * a.nParams + a.desc[c].paramOffset] = v;
    } else {
      bool bgParam = false;
      for (int c = 0; c < a.nComp; c++)
        if (a.desc[c].background && a.desc[c].paramOffset == j - 2) bgParam = true;
      if (!bgParam) a.grad[(long)b * a.nParams + (j - 2)] = v;
    }
  }
}

// Called by every thread of a CTA after its partials are written: the CTA
// that completes the evaluation's `total` CTAs for vector b performs the final
// reduction (threadfence-reduction pattern: no CTA waits for another).
__device__ __forceinline__ void finish_cta(const FastArgs &a, int b, int total, int nGradBlocks) {
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(a.done + b, 1u) == (unsigned)total - 1u);
  __syncthreads();
  if (last) {
    __threadfence();
    reduce_entry(a, b, nGradBlocks);
  }
}

// -------------------------- stat rows: c2r + statistic + g + g row r2c
// Per-pixel statistic term (FP32, accumulated per thread in FP32 over a few
// pixels; the block and final reductions are FP64) and its derivative
// g = dS/dM.  chi^2: (w (d - M))^2; with model-based errors
// (d - M)^2 / V(M), V = (M + sky)/g_eff + n_comb rn^2; Cash: 2 w (m' - d' ln m' + extra)
// with m' = g_eff (M + sky), ln m' replaced by 1e-25 when m' <= 0 (core/model_object.cpp:1703-1775).
__device__ __forceinline__ void stat_term(const FastArgs &a, long z, float m, float &S, float &gout) {
  const float cnt = a.count ? a.count[z] : 1.f;
  const float w = a.weight[z];
  if (cnt == 0.f || (w == 0.f && !a.modelErrors)) {
    gout = 0.f;
    return;
  }
  const float d = a.data[z];
  if (a.kind == 0) {
    if (a.modelErrors) {
      if (w <= 0.f) {  // masked
        gout = 0.f;
        return;
      }
      const float V = (m + a.sky) / a.effGain + a.rnTerm;
      const float r = d - m;
      S += cnt * r * r / V;
      gout = cnt * (-2.f * r / V - r * r / (V * V * a.effGain));
    } else {
      const float dev = w * (d - m);
      S += cnt * dev * dev;
      gout = -2.f * cnt * w * dev;
    }
  } else {
    const float mv = a.effGain * (m + a.sky);
    const float dv = a.effGain * (d + a.sky);
    const float ex = a.extra ? a.extra[z] : 0.f;
    float term, dterm;
    if (mv > 0.f) {
      if (ex != 0.f && dv > 0.f) {
        // (mv - dv ln mv) + (dv ln dv - dv) written without cancellation
        term = (mv - dv) - dv * log1pf((mv - dv) / dv);
      } else {
        term = mv - dv * logf(mv) + ex;
      }
      dterm = a.effGain * (1.f - dv / mv);
    } else {
      term = mv - dv * 1.0e-25f + ex;
      dterm = a.effGain;
    }
    S += 2.f * cnt * w * term;
    gout = 2.f * cnt * w * dterm;
  }
}

// CTA partial sums of (S, SG) into slot `slot` of vector b: FP32 over the
// thread's pixels and the warp, double-float across warps.  Every thread of
// the CTA calls it.
__device__ __forceinline__ void stat_partials(const FastArgs &a, int b, int slot, float S, float SG) {
  __shared__ ffloat red[2][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  S = warp_sum(S);
  SG = warp_sum(SG);
  if (lane == 0) {
    red[0][wid] = ff_make(S);
    red[1][wid] = ff_make(SG);
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    ffloat v0 = lane < nw ? red[0][lane] : ffloat{0.f, 0.f};
    ffloat v1 = lane < nw ? red[1][lane] : ffloat{0.f, 0.f};
    v0 = ff_warp_sum(v0);
    v1 = ff_warp_sum(v1);
    if (lane == 0) {
      float2 *p = a.statPart + (long)b * 2 * a.partStride + slot;
      p[0] = ff_store(v0);
      p[a.partStride] = ff_store(v1);
    }
  }
}

// ---------------------------------------- region: c2r + block average
// One CTA per replaced data row s of the oversampled region: the inverse row
// FFTs of its k subpixel rows and the k x k block averages.  mode 0: derivative
// images of the JtWJ pass (batch index b then runs over (parameter vector,
// parameter) pairs; no background; averages to `out`).  mode 1: the forward
// model -- background and point sources added -- and the statistic terms of
// the region's data pixels (the model image, when kept, gets their values);
// mode 2 adds their adjoint seeds g = dS/dM, spread as g / k^2 over the
// subpixels and row-transformed into the CTA's k rows of the region spectrum
// (the input of the adjoint column pass), and the point sources' derivative
// sums.  The statistic partials take the
// slots after the main window's (statBase + s); with doneTotal > 0 the last
// CTA of the evaluation adds them up.  The main window's statistic pass skips
// the region's pixels, so the two windows' pipelines share no dependency
// before the final reduction.
// PS: the model has point sources (their code is compiled only into the PS instance)
template <bool PS>
__global__ void __launch_bounds__(1024) k_fast_region_down(FastArgs a, FastGeom g, cplx<float> *__restrict__ rspec,
                                                          FFTPlan<float> plan, const cplx<float> *__restrict__ twL,
                                                          float *__restrict__ out, int mode, int statBase,
                                                          int doneTotal) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float psAcc[4 * kMaxPsFast];
  const int b = blockIdx.y, s = blockIdx.x;  // replaced data row within the region
  const int k = g.rScale;
  const int M = plan.n, ls = M + 1;
  cplx<float> *bufX = reinterpret_cast<cplx<float> *>(smem);
  cplx<float> *bufA = bufX + k * ls;
  cplx<float> *bufB = bufA + k * ls;
  if constexpr (PS)
    if (mode == 2)
      for (int i = threadIdx.x; i < 4 * a.nPs; i += blockDim.x) psAcc[i] = 0.f;
  cplx<float> *in = rspec + (long)b * g.rSpecBatch + (long)(s * k) * g.rSpecPitch;
  const FastDiv byM(M), byM1(M + 1);
  for (int idx = threadIdx.x; idx < k * (M + 1); idx += blockDim.x) {
    const int l = byM1.div(idx), kk = idx - l * (M + 1);
    bufX[l * ls + kk] = in[(long)l * g.rSpecPitch + kk];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < k * M; idx += blockDim.x) {
    const int l = byM.div(idx), kk = idx - l * M;
    bufA[l * ls + kk] = c2r_pre(bufX + l * ls, kk, M, twL);
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, plan, k, ls, 1, +1, false);
  pdl_trigger();
  const float inv = 1.f / (float)(k * k);
  if (mode == 0) {
    for (int t = threadIdx.x; t < g.rCols; t += blockDim.x) {
      float acc = 0.f;
      for (int u = 0; u < k; u++)
        for (int v = 0; v < k; v++) {
          const int col = t * k + v;
          const cplx<float> z = Z[u * ls + (col >> 1)];
          acc += (col & 1) ? z.y : z.x;
        }
      out[((long)b * g.rRows + s) * g.rCols + t] = acc * inv;
    }
    return;
  }
  if (a.dataStride) {  // image stack: this entry's data and weights
    const long img = a.entry ? a.entry[b] : b;
    a.data += img * a.dataStride;
    a.weight += img * a.dataStride;
  }
  if (a.count && a.countStride) a.count += (a.entry ? a.entry[b] : b) * a.countStride;  // batched bootstrap
  const float bg = a.bgLevel[2 * b + 1];
  const int row = g.ry0 + s;
  float *gRow = reinterpret_cast<float *>(bufX);  // the loaded spectrum is consumed
  float S = 0.f, SG = 0.f;
  for (int t = threadIdx.x; t < g.rCols; t += blockDim.x) {
    float acc = 0.f;
    for (int u = 0; u < k; u++)
      for (int v = 0; v < k; v++) {
        const int col = t * k + v;
        const cplx<float> z = Z[u * ls + (col >> 1)];
        acc += (col & 1) ? z.y : z.x;
      }
    const int col = g.rx0 + t;
    if constexpr (PS) acc += ps_region(a, k, b, row, col, 0.f, nullptr);
    const float m = acc * inv + bg;
    const long zi = (long)row * g.nDataCols + col;
    if (a.modelOut) a.modelOut[(long)b * g.nDataRows * g.nDataCols + zi] = m;
    float gz;
    stat_term(a, zi, m, S, gz);
    SG += gz * a.psfSumOs;
    if (mode == 2) {
      if constexpr (PS)
        if (gz != 0.f) ps_region(a, k, b, row, col, gz * inv, psAcc);
      gRow[t] = gz;
    }
  }
  stat_partials(a, b, statBase + s, S, SG);  // (its barrier also publishes gRow)
  if (mode == 2) {
    // adjoint seed: g / k^2 on each of the row's k x k subpixels.  Its k
    // subpixel rows are equal, so one r2c serves all k rows of the region
    // spectrum (those this CTA read above).
    cplx<float> *G = (Z == bufA) ? bufB : bufA;
    const float invk = 1.f / (float)k;
    for (int kk = threadIdx.x; kk < M; kk += blockDim.x) {
      const int c0 = 2 * kk, c1 = 2 * kk + 1;
      cplx<float> z;
      z.x = (c0 < g.rSubCols) ? gRow[floordiv_scale(c0, invk)] * inv : 0.f;
      z.y = (c1 < g.rSubCols) ? gRow[floordiv_scale(c1, invk)] * inv : 0.f;
      G[kk] = z;
    }
    __syncthreads();
    cplx<float> *R = block_fft(G, Z, plan, 1, ls, 1, -1, false);
    for (int kk = threadIdx.x; kk <= M; kk += blockDim.x) {
      const cplx<float> v = r2c_post(R, kk, M, twL);
      for (int u = 0; u < k; u++) in[(long)u * g.rSpecPitch + kk] = v;
    }
  }
  if constexpr (PS) {
    if (mode == 2) {
      __syncthreads();
      for (int i = threadIdx.x; i < 4 * a.nPs; i += blockDim.x)
        a.psPart[((long)b * 4 * a.nPs + i) * a.partStride + statBase + s] = make_float2(psAcc[i], 0.f);
    }
  }
  if (doneTotal > 0) finish_cta(a, b, doneTotal, 0);
}

template <bool PS>
__global__ void __launch_bounds__(1024) k_fast_stat_rows(FastArgs a, FastGeom g, FFTPlan<float> plan,
                                                        const cplx<float> *__restrict__ twL, int rpb, int wantGrad,
                                                        int doneTotal) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y;
  const int M = plan.n, ls = M + 1;
  cplx<float> *bufX = reinterpret_cast<cplx<float> *>(smem);
  cplx<float> *bufA = bufX + rpb * ls;
  cplx<float> *bufB = bufA + rpb * ls;
  __shared__ float psAcc[4 * kMaxPsFast];
  if constexpr (PS)
    for (int i = threadIdx.x; i < 4 * a.nPs; i += blockDim.x) psAcc[i] = 0.f;
  const int row0 = blockIdx.x * rpb;
  const int nl = min(rpb, g.nDataRows - row0);
  cplx<float> *spec = reinterpret_cast<cplx<float> *>(a.spec) + (long)b * g.specBatch;
  float S = 0.f, SG = 0.f;
  if (a.dataStride) {  // image stack: this entry's data and weights
    const long img = a.entry ? a.entry[b] : b;
    a.data += img * a.dataStride;
    a.weight += img * a.dataStride;
  }
  if (a.count && a.countStride) a.count += (a.entry ? a.entry[b] : b) * a.countStride;  // batched bootstrap
  const FastDiv byM(M), byM1(M + 1);
  if (nl > 0) {
    for (int idx = threadIdx.x; idx < nl * (M + 1); idx += blockDim.x) {
      const int l = byM1.div(idx), k = idx - l * (M + 1);
      bufX[l * ls + k] = spec[(long)(row0 + l) * g.specPitch + k];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
      const int l = byM.div(idx), k = idx - l * M;
      bufA[l * ls + k] = c2r_pre(bufX + l * ls, k, M, twL);
    }
    __syncthreads();
    cplx<float> *Z = block_fft(bufA, bufB, plan, nl, ls, 1, +1, false);
    cplx<float> *G = (Z == bufA) ? bufB : bufA;
    const float bg = a.bgLevel[2 * b];
    // one thread per complex point = two data columns
    for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
      const int l = byM.div(idx), k = idx - l * M;
      const int row = row0 + l;
      const cplx<float> zz = Z[l * ls + k];
      float gv[2] = {0.f, 0.f};
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const int col = 2 * k + e;
        if (col >= g.nDataCols) continue;
        const long zi = (long)row * g.nDataCols + col;
        if (g.hasRegion) {  // the region's pixels: k_fast_region_down
          const int rr = row - g.ry0, rc = col - g.rx0;
          if (rr >= 0 && rr < g.rRows && rc >= 0 && rc < g.rCols) continue;
        }
        float m = (e ? zz.y : zz.x) + bg;
        if constexpr (PS) m += ps_main(a, b, row, col, 0.f, nullptr);
        if (a.modelOut) a.modelOut[(long)b * g.nDataRows * g.nDataCols + zi] = m;
        float gz;
        stat_term(a, zi, m, S, gz);
        SG += gz * a.psfSum;
        if constexpr (PS)
          if (wantGrad && gz != 0.f) ps_main(a, b, row, col, gz, psAcc);
        gv[e] = gz;
      }
      G[l * ls + k] = {gv[0], gv[1]};
    }
    __syncthreads();
    if (wantGrad) {
      cplx<float> *other = (G == bufA) ? bufB : bufA;
      cplx<float> *R = block_fft(G, other, plan, nl, ls, 1, -1, false);
      for (int idx = threadIdx.x; idx < nl * (M + 1); idx += blockDim.x) {
        const int l = byM1.div(idx), k = idx - l * (M + 1);
        spec[(long)(row0 + l) * g.specPitch + k] = r2c_post(R + l * ls, k, M, twL);
      }
    }
  }
  pdl_trigger();
  stat_partials(a, b, blockIdx.x, S, SG);
  if constexpr (PS) {
    if (wantGrad) {
      __syncthreads();
      for (int i = threadIdx.x; i < 4 * a.nPs; i += blockDim.x)
        a.psPart[((long)b * 4 * a.nPs + i) * a.partStride + blockIdx.x] = make_float2(psAcc[i], 0.f);
    }
  }
  if (doneTotal > 0) finish_cta(a, b, doneTotal, 0);
}

// ---------------------------------------- gradient pass over the window
// acc[0..1+NP] += r~ * dm/dtheta over the CTA's window pixels for component cc
// (X0, Y0, then its function parameters); subsampled pixels from the table.
template <int TY, bool REG, bool BOX>
__device__ __forceinline__ void grad_pixels(const CompF32 cc, const WinDesc &w, const float *rt, int ls, int row0,
                                            int npix, const FastDiv &byCols, const float *tab, int side, int bc0,
                                            int br0, float *acc) {
  constexpr int NP = n_fparams<TY>();
  float o[7];
  for (int idx = threadIdx.x; idx < npix; idx += blockDim.x) {
    const int l = byCols.div(idx), col = idx - l * w.cols;
    const int row = row0 + l;
    const float r = rt[2 * l * ls + col];
    float dx, dy;
    win_offsets_t<REG>(w, cc, row, col, dx, dy);
    if constexpr (TY == F_TILTEDSKY) {
      if (r == 0.f) continue;
      plane_grad32(cc, dx, dy, r, o);
    } else {
      const Geo g = geo32(cc, dx, dy);
      if (BOX && subsampling_t<TY>() && g.r2 < 100.f) {
        const int ns = n_subsamples32(cc, fast_sqrt(g.r2));
        if (ns > 1) {
          const int br = row - br0, bc = col - bc0;
          if (br >= 0 && br < side && bc >= 0 && bc < side) {
            const float *t = tab + ((long)br * side + bc) * 8 + 1;
#pragma unroll
            for (int q = 0; q < 2 + NP; q++) acc[q] += r * t[q];
          } else {
            // outside the precomputed box (not reached for radius < 10): direct average
            const float d = 1.f / ns;
            for (int t = 0; t < ns * ns; t++) {
              const Geo gs = geo32(cc, dx - 0.5f + (t / ns + 0.5f) * d, dy - 0.5f + (t % ns + 0.5f) * d);
              radial_grad_t<TY>(cc, gs, r * d * d, o);
#pragma unroll
              for (int q = 0; q < 2 + NP; q++) acc[q] += o[q];
            }
          }
          continue;
        }
      }
      if (r == 0.f) continue;
      radial_grad_t<TY>(cc, g, r, o);
    }
#pragma unroll
    for (int q = 0; q < 2 + NP; q++) acc[q] += o[q];
  }
}

template <int TY>
__device__ __forceinline__ void grad_pixels_rt(bool reg, bool box, const CompF32 &cc, const WinDesc &w,
                                               const float *rt, int ls, int row0, int npix, const FastDiv &byCols,
                                               const float *tab, int side, int bc0, int br0, float *acc) {
  if (reg) {
    if (box) grad_pixels<TY, true, true>(cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc);
    else grad_pixels<TY, true, false>(cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc);
  } else {
    if (box) grad_pixels<TY, false, true>(cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc);
    else grad_pixels<TY, false, false>(cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc);
  }
}

__global__ void __launch_bounds__(1024) k_fast_grad_rows(FastArgs a, WinDesc w, FFTPlan<float> plan,
                                                        const cplx<float> *__restrict__ twL, int rpb,
                                                        float2 *__restrict__ gradPart, int blockBase, int win,
                                                        int doneTotal) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y;
  const int M = plan.n, ls = M + 1;
  CompF32 *sc = reinterpret_cast<CompF32 *>(smem);
  int *boxes = reinterpret_cast<int *>(sc + kMaxComponents);
  cplx<float> *bufX = reinterpret_cast<cplx<float> *>(boxes + 2 * kMaxComponents);
  cplx<float> *bufA = bufX + rpb * ls;
  cplx<float> *bufB = bufA + rpb * ls;
  // per-warp double-float sums of every parameter's term over the
  // components: [warp][parameter]; added across warps once, at the end
  ffloat *wpart = reinterpret_cast<ffloat *>(bufB + rpb * ls);
  const int nC = a.nComp, nP = a.nParams;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) {
    sc[i] = a.comps[b * nC + i];
    const int *o = a.subBox + (((long)b * nC + i) * 2 + win) * 2;
    boxes[2 * i] = o[0];
    boxes[2 * i + 1] = o[1];
  }
  for (int i = threadIdx.x; i < (blockDim.x >> 5) * nP; i += blockDim.x) wpart[i] = ffloat{0.f, 0.f};
  const int row0 = blockIdx.x * rpb;
  const int nl = min(rpb, w.rows - row0);
  const cplx<float> *spec = w.spec + (long)b * w.specBatch;
  const FastDiv byM(M), byM1(M + 1), byCols(w.cols);
  for (int idx = threadIdx.x; idx < max(nl, 0) * (M + 1); idx += blockDim.x) {
    const int l = byM1.div(idx), k = idx - l * (M + 1);
    bufX[l * ls + k] = spec[(long)(row0 + l) * w.specPitch + k];
  }
  __syncthreads();
  if (nl > 0) {
    for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
      const int l = byM.div(idx), k = idx - l * M;
      bufA[l * ls + k] = c2r_pre(bufX + l * ls, k, M, twL);
    }
    __syncthreads();
    cplx<float> *Z = block_fft(bufA, bufB, plan, nl, ls, 1, +1, false);
    const float *rt = reinterpret_cast<const float *>(Z);  // r~ of (l, col) at rt[2*(l*ls) + col]
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int npix = nl * w.cols;
    if (w.losRt)
      for (int idx = threadIdx.x; idx < npix; idx += blockDim.x) {
        const int l = byCols.div(idx), col = idx - l * w.cols;
        w.losRt[((long)b * w.rows + row0 + l) * w.cols + col] = rt[2 * l * ls + col];
      }
    for (int c = 0; c < nC; c++) {
      const CompF32 cc = sc[c];
      if (!in_rows(cc.type)) continue;
      const int side = win ? a.boxReg : a.boxMain;
      const float *tab = a.subTab + sub_base(a, b, c, win);
      const int bc0 = boxes[2 * c], br0 = boxes[2 * c + 1];
      const bool box = rows_meet_box(cc, row0, nl, br0, side);
      float acc[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      switch (cc.type) {
        case F_SERSIC: grad_pixels_rt<F_SERSIC>(w.isRegion, box, cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc); break;
        case F_EXP: grad_pixels_rt<F_EXP>(w.isRegion, box, cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc); break;
        case F_GRING: grad_pixels_rt<F_GRING>(w.isRegion, box, cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc); break;
        case F_MOFFAT: grad_pixels_rt<F_MOFFAT>(w.isRegion, box, cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc); break;
        case F_GAUSS: grad_pixels_rt<F_GAUSS>(w.isRegion, box, cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc); break;
        case F_TILTEDSKY:
          grad_pixels_rt<F_TILTEDSKY>(w.isRegion, box, cc, w, rt, ls, row0, npix, byCols, tab, side, bc0, br0, acc);
          break;
        default: break;
      }
      // FP32 over the warp, then into the warp's double-float parameter sums
      // (no barrier: each warp owns its row of wpart)
#pragma unroll
      for (int q = 0; q < 7; q++) acc[q] = warp_sum(acc[q]);
      if (lane == 0) {
        const int npf = a.desc[c].nParams;
        ffloat *wp = wpart + wid * nP;
#pragma unroll
        for (int q = 0; q < 7; q++) {
          const int slot = q == 0 ? cc.x0Index : q == 1 ? cc.x0Index + 1 : (q - 2 < npf ? cc.paramOffset + q - 2 : -1);
          if (slot >= 0) wp[slot] = ff_add(wp[slot], ff_make(acc[q]));
        }
      }
    }
  }
  __syncthreads();
  pdl_trigger();
  // CTA partials: double-float across the warps, in warp order
  const int nw = blockDim.x >> 5;
  float2 *out = gradPart + (long)b * nP * a.partStride + blockBase + blockIdx.x;
  for (int i = threadIdx.x; i < nP; i += blockDim.x) {
    ffloat t = {0.f, 0.f};
    for (int v = 0; v < nw; v++) t = ff_add(t, wpart[v * nP + i]);
    out[(long)i * a.partStride] = ff_store(t);
  }
  if (doneTotal > 0) finish_cta(a, b, doneTotal, doneTotal);
}

// ------------------------------------------------- 3-D line-of-sight terms
// Rotated-frame coordinates of a window pixel for a component.
__device__ __forceinline__ void los_pixel(const WinDesc &w, const CompF32 &cc, int row, int col, float &xp,
                                          float &yp) {
  float dx, dy;
  win_offsets(w, cc, row, col, dx, dy);
  xp = fmaf(dx, cc.cosPA, dy * cc.sinPA);
  yp = fmaf(-dx, cc.sinPA, dy * cc.cosPA);
}

// Kept partitions: [B][nLos][window pixels][32] panels (lo, hi) and the panel
// counts, so the gradient pass integrates the derivatives over the forward
// pass's panels instead of searching again.
struct LosStore {
  float2 *panels;
  int *count;
  int nLos;
};

// index of component c among the model's 3-D components
__device__ __forceinline__ int los_index(const CompF32 *sc, int c) {
  int k = 0;
  for (int i = 0; i < c; i++) k += is_los(sc[i].type);
  return k;
}

// One warp per window pixel (grid-stride): sum of the 3-D components' line of
// sight integrals, written to w.losVal (added to the model row by eval_r2c);
// with a store, each partition is kept for the gradient pass.
__global__ void __launch_bounds__(256) k_fast_los_eval(FastArgs a, WinDesc w, LosStore ks) {
  pdl_wait();
  __shared__ CompF32 sc[kMaxComponents];
  const int b = blockIdx.y;
  const int nC = a.nComp;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) sc[i] = a.comps[b * nC + i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const GkLane nd = gk21_lane();
  const long npix = (long)w.rows * w.cols;
  const long nWarps = (long)gridDim.x * (blockDim.x >> 5);
  for (long p = blockIdx.x * (long)(blockDim.x >> 5) + (threadIdx.x >> 5); p < npix; p += nWarps) {
    const int row = (int)(p / w.cols), col = (int)(p - (long)row * w.cols);
    float v = 0.f;
    for (int c = 0; c < nC; c++) {
      const CompF32 &cc = sc[c];
      if (!is_los(cc.type)) continue;
      float xp, yp;
      los_pixel(w, cc, row, col, xp, yp);
      float lo, hi, total;
      const int np = los_partition(cc, xp, yp, nd, lo, hi, total);
      v += total;
      if (ks.panels) {
        const long slot = ((long)b * ks.nLos + los_index(sc, c)) * npix + p;
        if (lane < np) ks.panels[slot * 32 + lane] = make_float2(lo, hi);
        if (lane == 0) ks.count[slot] = np;
      }
    }
    if (lane == 0) w.losVal[(long)b * npix + p] = v;
  }
}

// One warp per window pixel: r~ * d(line-of-sight value)/d(parameters) of
// every 3-D component, per-warp rows in shared memory (no atomics), then one
// FP32 partial per parameter for this CTA.
// four CTAs per SM (64 registers): the measured optimum for the gradient pass
__global__ void __launch_bounds__(256, 4) k_fast_los_grad(FastArgs a, WinDesc w, float2 *__restrict__ gradPart,
                                                      int blockBase, LosStore ks, int doneTotal) {
  pdl_wait();
  __shared__ CompF32 sc[kMaxComponents];
  __shared__ float red[8][kMaxParams];
  const int b = blockIdx.y;
  const int nC = a.nComp, nP = a.nParams;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) sc[i] = a.comps[b * nC + i];
  for (int i = threadIdx.x; i < 8 * kMaxParams; i += blockDim.x) (&red[0][0])[i] = 0.f;
  __syncthreads();
  const GkLane nd = gk21_lane();
  const long npix = (long)w.rows * w.cols;
  const long nWarps = (long)gridDim.x * (blockDim.x >> 5);
  for (long p = blockIdx.x * (long)(blockDim.x >> 5) + wid; p < npix; p += nWarps) {
    const float r = w.losRt[(long)b * npix + p];
    if (r == 0.f) continue;
    const int row = (int)(p / w.cols), col = (int)(p - (long)row * w.cols);
    for (int c = 0; c < nC; c++) {
      const CompF32 &cc = sc[c];
      if (!is_los(cc.type)) continue;
      float xp, yp, g[kLosGrad];
      los_pixel(w, cc, row, col, xp, yp);
      if (ks.panels) {
        const long slot = ((long)b * ks.nLos + los_index(sc, c)) * npix + p;
        const int np = ks.count[slot];
        const float2 pn = lane < np ? ks.panels[slot * 32 + lane] : make_float2(0.f, 0.f);
        los_grad_panels(cc, xp, yp, nd, np, pn.x, pn.y, g);
      } else {
        los_grad_warp(cc, xp, yp, nd, g);
      }
      if (lane == 0) {
        red[wid][cc.x0Index] += r * g[0];
        red[wid][cc.x0Index + 1] += r * g[1];
        const int npf = los_nparams(cc);
        for (int q = 0; q < npf; q++) red[wid][cc.paramOffset + q] += r * g[2 + q];
      }
    }
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  for (int j = threadIdx.x; j < nP; j += blockDim.x) {
    ffloat t = {0.f, 0.f};
    for (int i = 0; i < nw; i++) t = ff_add(t, red[i][j]);
    gradPart[((long)b * nP + j) * a.partStride + blockBase + blockIdx.x] = ff_store(t);
  }
  if (doneTotal > 0) finish_cta(a, b, doneTotal, doneTotal);
}

// ------------------------------------------------------------- reduce
// One CTA per output quantity (statistic, background term, each gradient
// entry): FP64 sum of the per-CTA FP32 partials in a fixed order.
__device__ __forceinline__ double block_sum_d(double v) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum_d(v);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    v = lane < nw ? sh[lane] : 0.0;
    v = warp_sum_d(v);
  }
  return v;
}

// ------------------------------------ forward-mode derivative images (JtWJ)
// Adds component cc's dm/dtheta at every pixel of window row `row` to the
// derivative lines sl[q] (q: X0, Y0, then its function parameters; -1 = not
// a derivative line); each column belongs to one thread.
template <int TY, bool REG, bool BOX>
__device__ __forceinline__ void deriv_pixels(const CompF32 cc, const WinDesc &w, int row, const int *sl,
                                             float *lines, int ls, const float *tab, int side, int bc0, int br0) {
  constexpr int NP = n_fparams<TY>();
  for (int col = threadIdx.x; col < w.cols; col += blockDim.x) {
    float dx, dy;
    win_offsets_t<REG>(w, cc, row, col, dx, dy);
    float o[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if constexpr (TY == F_TILTEDSKY) {
      plane_grad32(cc, dx, dy, 1.f, o);
    } else {
      const Geo g = geo32(cc, dx, dy);
      const int ns = (BOX && subsampling_t<TY>() && g.r2 < 100.f) ? n_subsamples32(cc, fast_sqrt(g.r2)) : 1;
      if (ns > 1) {
        const int br = row - br0, bc = col - bc0;
        if (br >= 0 && br < side && bc >= 0 && bc < side) {
          const float *t = tab + ((long)br * side + bc) * 8 + 1;
#pragma unroll
          for (int q = 0; q < 2 + NP; q++) o[q] = t[q];
        } else {
          // outside the precomputed box (not reached for radius < 10): direct average
          const float d = 1.f / ns;
          float t7[7];
          for (int t = 0; t < ns * ns; t++) {
            const Geo gs = geo32(cc, dx - 0.5f + (t / ns + 0.5f) * d, dy - 0.5f + (t % ns + 0.5f) * d);
            radial_grad_t<TY>(cc, gs, d * d, t7);
#pragma unroll
            for (int q = 0; q < 2 + NP; q++) o[q] += t7[q];
          }
        }
      } else {
        radial_grad_t<TY>(cc, g, 1.f, o);
      }
    }
#pragma unroll
    for (int q = 0; q < 2 + NP; q++)
      if (sl[q] >= 0) lines[2 * sl[q] * ls + col] += o[q];
  }
}

template <int TY>
__device__ __forceinline__ void deriv_pixels_rt(bool reg, bool box, const CompF32 &cc, const WinDesc &w, int row,
                                                const int *sl, float *lines, int ls, const float *tab, int side,
                                                int bc0, int br0) {
  if (reg) {
    if (box) deriv_pixels<TY, true, true>(cc, w, row, sl, lines, ls, tab, side, bc0, br0);
    else deriv_pixels<TY, true, false>(cc, w, row, sl, lines, ls, tab, side, bc0, br0);
  } else {
    if (box) deriv_pixels<TY, false, true>(cc, w, row, sl, lines, ls, tab, side, bc0, br0);
    else deriv_pixels<TY, false, false>(cc, w, row, sl, lines, ls, tab, side, bc0, br0);
  }
}

// One CTA per (window row, parameter vector): dm/dtheta_j of every
// non-background parameter at every pixel of the row -- analytic, subsampled
// pixels from the precomputed table -- accumulated into nD real lines in
// shared memory (a pixel belongs to one thread, so no atomics), then the nD
// row FFTs.  Derivative spectra of parameter vector b are the nD consecutive
// entries b*nD .. b*nD+nD-1 of the spectrum batch.
__global__ void __launch_bounds__(512) k_fast_deriv_r2c(FastArgs a, WinDesc w, FFTPlan<float> plan,
                                                        const cplx<float> *__restrict__ twL,
                                                        const int *__restrict__ slot, int nD, int win) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y, row = blockIdx.x;
  const int M = plan.n, ls = M + 1;
  CompF32 *sc = reinterpret_cast<CompF32 *>(smem);
  int *boxes = reinterpret_cast<int *>(sc + kMaxComponents);
  int *npar = boxes + 2 * kMaxComponents;
  int *ss = npar + kMaxComponents;
  cplx<float> *bufA = reinterpret_cast<cplx<float> *>(ss + kMaxParams);
  cplx<float> *bufB = bufA + nD * ls;
  const int nC = a.nComp;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) {
    sc[i] = a.comps[b * nC + i];
    const int *o = a.subBox + (((long)b * nC + i) * 2 + win) * 2;
    boxes[2 * i] = o[0];
    boxes[2 * i + 1] = o[1];
    npar[i] = a.desc[i].nParams;
  }
  for (int i = threadIdx.x; i < a.nParams; i += blockDim.x) ss[i] = slot[i];
  for (int i = threadIdx.x; i < nD * ls; i += blockDim.x) bufA[i] = {0.f, 0.f};
  __syncthreads();
  float *lines = reinterpret_cast<float *>(bufA);  // real line j: lines[2 * j * ls + col]
  const int side = win ? a.boxReg : a.boxMain;
  for (int c = 0; c < nC; c++) {
    const CompF32 cc = sc[c];
    if (!in_rows(cc.type)) continue;
    // the derivative lines this component's parameters feed (-1: none)
    int sl[7];
    sl[0] = ss[cc.x0Index];
    sl[1] = ss[cc.x0Index + 1];
#pragma unroll
    for (int q = 0; q < 5; q++) sl[2 + q] = q < npar[c] ? ss[cc.paramOffset + q] : -1;
    const float *tab = a.subTab + sub_base(a, b, c, win);
    const int bc0 = boxes[2 * c], br0 = boxes[2 * c + 1];
    const bool box = rows_meet_box(cc, row, 1, br0, side);
    switch (cc.type) {
      case F_SERSIC: deriv_pixels_rt<F_SERSIC>(w.isRegion, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_EXP: deriv_pixels_rt<F_EXP>(w.isRegion, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_GRING: deriv_pixels_rt<F_GRING>(w.isRegion, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_MOFFAT: deriv_pixels_rt<F_MOFFAT>(w.isRegion, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_GAUSS: deriv_pixels_rt<F_GAUSS>(w.isRegion, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_TILTEDSKY: deriv_pixels_rt<F_TILTEDSKY>(w.isRegion, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      default: break;
    }
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, plan, nD, ls, 1, -1, false);
  cplx<float> *out = w.spec + (long)b * nD * w.specBatch + (long)row * w.specPitch;
  const FastDiv byM1(M + 1);
  for (int idx = threadIdx.x; idx < nD * (M + 1); idx += blockDim.x) {
    const int j = byM1.div(idx), k = idx - j * (M + 1);
    out[(long)j * w.specBatch + k] = r2c_post(Z + j * ls, k, M, twL);
  }
}

// Deviate of pixel z at model value m and its slope q = d(deviate)/dM, so the
// Levenberg-Marquardt Jacobian is J_zj = q_z dM_z/dtheta_j.
//   chi^2, data/external errors: dev = w (d - M)               (model_object.cpp:1480-1490)
//   chi^2, model errors:         dev = (d - M) / sqrt(V(M))    (model_object.cpp:1345-1381)
//   Poisson-MLR:                 dev = sqrt(2 w |m' - d' ln m' + extra|)  (model_object.cpp:1386-1401)
__device__ __forceinline__ void deviate_slope(const FastArgs &a, long z, float m, float &dev, float &q) {
  const float w = a.weight[z];
  dev = 0.f;
  q = 0.f;
  if (a.kind == 0) {
    if (a.modelErrors) {
      if (w <= 0.f) return;
      const float V = (m + a.sky) / a.effGain + a.rnTerm;
      const float iv = 1.f / sqrtf(V);
      const float r = a.data[z] - m;
      dev = r * iv;
      q = -iv - 0.5f * r * iv / (V * a.effGain);
    } else {
      dev = w * (a.data[z] - m);
      q = -w;
    }
    return;
  }
  if (w == 0.f) return;
  const float mv = a.effGain * (m + a.sky), dv = a.effGain * (a.data[z] + a.sky);
  const float ex = a.extra ? a.extra[z] : 0.f;
  float T, dT;
  if (mv > 0.f) {
    T = (ex != 0.f && dv > 0.f) ? (mv - dv) - dv * log1pf((mv - dv) / dv) : mv - dv * logf(mv) + ex;
    dT = a.effGain * (1.f - dv / mv);
  } else {
    T = mv - dv * 1.0e-25f + ex;
    dT = a.effGain;
  }
  dev = sqrtf(2.f * w * fabsf(T));
  q = (dev > 0.f) ? ((T < 0.f) ? -1.f : 1.f) * w * dT / dev : 0.f;
}

// Row partial sums of J^T W J as the upper triangle of one augmented Gram
// matrix: with a_j (j < nP) the Jacobian rows of the deviates, a_nP = dev and
// c the pixel weights (bootstrap multiplicities; W = false: all 1),
//   G = sum over the row's columns of c a a^T,
// G_jk (j <= k < nP) = alpha_jk, G_j,nP = beta_j, G_nP,nP = S, stored in the
// order alpha (row-major upper triangle), beta, S.  Warps take 4 x 4 tiles of
// the triangle over one chunk of the columns (lanes on consecutive columns:
// conflict-free shared loads, 16 FMAs per 8 loads), reduce each tile entry
// across the warp (FP32: at most 32 partial sums), and the chunks' sums are
// added in a fixed order in double-float, stored as (hi, lo) pairs.
// Row j of a is at U + ss[j] * uStride (ss[j] < 0: the background row qb),
// row nP at dv, rows past nP at zero (nc zeros).  red holds jtwj_splits() x Q
// floats.  All threads of the CTA call it; ends with a barrier.
__host__ __device__ inline int jtwj_tiles(int nP) {
  const int nt = (nP + 4) / 4;  // tiles per side of the (nP + 1)^2 matrix
  return nt * (nt + 1) / 2;
}
__host__ __device__ inline int jtwj_splits(int nP, int threads) {
  const int s = 4 * (threads / 32) / jtwj_tiles(nP);
  return s < 1 ? 1 : (s > 16 ? 16 : s);
}
__host__ __device__ inline int jtwj_aux_floats(int nP, int nc, int threads) {
  const int Q = nP * (nP + 1) / 2 + nP + 1;
  return 4 * nc + jtwj_splits(nP, threads) * Q;
}

template <bool W>
__device__ __forceinline__ void jtwj_gram(const float *U, long uStride, const int *ss, const float *qb,
                                          const float *dv, const float *zero, const float *cw, int nc, int nP,
                                          float *red, float2 *out, long outStride) {
  const int n1 = nP + 1, nt = (n1 + 3) / 4, nTiles = nt * (nt + 1) / 2;
  const int nPair = nP * (nP + 1) / 2, Q = nPair + nP + 1;
  const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nSplit = jtwj_splits(nP, blockDim.x);
  const int chunk = (((nc + nSplit - 1) / nSplit) + 31) & ~31;
  for (int item = warp; item < nTiles * nSplit; item += nw) {
    const int sp = item / nTiles;
    int I = 0, r = item - sp * nTiles;
    while (r >= nt - I) {
      r -= nt - I;
      I++;
    }
    const int J = I + r;
    const float *X[4], *Y[4];
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const int jx = 4 * I + t, jy = 4 * J + t;
      X[t] = jx < nP ? (ss[jx] >= 0 ? U + ss[jx] * uStride : qb) : (jx == nP ? dv : zero);
      Y[t] = jy < nP ? (ss[jy] >= 0 ? U + ss[jy] * uStride : qb) : (jy == nP ? dv : zero);
    }
    float acc[4][4];
#pragma unroll
    for (int t = 0; t < 4; t++)
#pragma unroll
      for (int u = 0; u < 4; u++) acc[t][u] = 0.f;
    const int c1 = min(nc, (sp + 1) * chunk);
    for (int col = sp * chunk + lane; col < c1; col += 32) {
      float x[4], y[4];
      const float c = W ? cw[col] : 1.f;
#pragma unroll
      for (int t = 0; t < 4; t++) {
        x[t] = W ? X[t][col] * c : X[t][col];
        y[t] = Y[t][col];
      }
#pragma unroll
      for (int t = 0; t < 4; t++)
#pragma unroll
        for (int u = 0; u < 4; u++) acc[t][u] = fmaf(x[t], y[u], acc[t][u]);
    }
#pragma unroll
    for (int t = 0; t < 4; t++)
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int j = 4 * I + t, k = 4 * J + u;
        if (j > k || k >= n1) continue;  // uniform across the warp
        const float v = warp_sum(acc[t][u]);
        if (lane == 0) {
          const int qi = k < nP ? j * nP - j * (j - 1) / 2 + (k - j) : (j < nP ? nPair + j : nPair + nP);
          red[sp * Q + qi] = v;
        }
      }
  }
  __syncthreads();
  for (int qi = threadIdx.x; qi < Q; qi += blockDim.x) {
    ffloat t = ff_make(0.f);  // the chunks' warp sums, added in double-float
    for (int sp = 0; sp < nSplit; sp++) t = ff_add(t, red[sp * Q + qi]);
    out[qi * outStride] = ff_store(t);
  }
}

// One CTA per (data row, parameter vector): inverse row FFT of the nD
// convolved derivative rows, the per-pixel Jacobian rows u_j = q dM/dtheta_j
// (region pixels from the downsampled region derivatives, background
// parameters from sum(PSF)), then the row's partial sums of
//   alpha_jk = sum c u_j u_k (j <= k),  beta_j = sum c u_j dev,  S = sum c dev^2
// (c = bootstrap multiplicity) in FP32, one partial per quantity per CTA.
template <bool PS>
__global__ void __launch_bounds__(1024) k_fast_jtwj_rows(FastArgs a, FastGeom g, FFTPlan<float> plan,
                                                        const cplx<float> *__restrict__ twL,
                                                        const cplx<float> *__restrict__ dspec,
                                                        const float *__restrict__ regDeriv,
                                                        const int *__restrict__ slot, int nD,
                                                        float2 *__restrict__ part, float *__restrict__ jac) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y, row = blockIdx.x;
  const int M = plan.n, ls = M + 1, nP = a.nParams, nc = g.nDataCols;
  int *ss = reinterpret_cast<int *>(smem);
  cplx<float> *bufA = reinterpret_cast<cplx<float> *>(ss + kMaxParams);
  cplx<float> *bufB = bufA + nD * ls;
  for (int i = threadIdx.x; i < nP; i += blockDim.x) ss[i] = slot[i];
  if (a.dataStride) {  // image stack: this entry's data and weights
    const long img = a.entry ? a.entry[b] : b;
    a.data += img * a.dataStride;
    a.weight += img * a.dataStride;
  }
  if (a.count && a.countStride) a.count += (a.entry ? a.entry[b] : b) * a.countStride;  // batched bootstrap
  const cplx<float> *src = dspec + (long)b * nD * g.specBatch + (long)row * g.specPitch;
  const FastDiv byM(M);
  for (int idx = threadIdx.x; idx < nD * M; idx += blockDim.x) {
    const int j = byM.div(idx), k = idx - j * M;
    bufA[j * ls + k] = c2r_pre(src + (long)j * g.specBatch, k, M, twL);
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, plan, nD, ls, 1, +1, false);
  // the Jacobian rows overwrite the real rows they are formed from (row j at
  // Zr + 2 j ls); the per-pixel vectors and the chunk sums use the other FFT
  // buffer when they fit there, else the space after bufB
  float *Zr = reinterpret_cast<float *>(Z);
  const long uStride = 2L * ls;
  float *aux = (jtwj_aux_floats(nP, nc, blockDim.x) <= 2 * nD * ls)
                   ? reinterpret_cast<float *>(Z == bufA ? bufB : bufA)
                   : reinterpret_cast<float *>(bufB + nD * ls);
  float *qb = aux, *cw = qb + nc, *dv = cw + nc, *zero = dv + nc, *red = zero + nc;
  const long nPix = (long)g.nDataRows * nc;
  for (int col = threadIdx.x; col < nc; col += blockDim.x) {
    const long zi = (long)row * nc + col;
    const float m = a.modelOut[(long)b * nPix + zi];
    float dev, q;
    deviate_slope(a, zi, m, dev, q);
    const float cnt = a.count ? a.count[zi] : 1.f;
    bool inReg = false;
    long ri = 0;
    if (g.hasRegion) {
      const int rr = row - g.ry0, rc = col - g.rx0;
      if (rr >= 0 && rr < g.rRows && rc >= 0 && rc < g.rCols) {
        inReg = true;
        ri = (long)rr * g.rCols + rc;
      }
    }
    const long rStride = (long)g.rRows * g.rCols;
    for (int j = 0; j < nD; j++) {
      float *u = Zr + j * uStride + col;
      *u = q * (inReg ? regDeriv[((long)b * nD + j) * rStride + ri] : *u);
    }
    for (int ps = 0; PS && ps < a.nPs; ps++) {  // point sources: derivatives after the convolution
      const CompF32 &c = a.comps[b * a.nComp + a.psComp[ps]];
      const CompDesc &d = a.desc[a.psComp[ps]];
      float dsum[4] = {0.f, 0.f, 0.f, 0.f};
      float X, Y;
      ps_offsets(c, row, col, X, Y);
      if (inReg) {
        const int k = g.rScale;
        const float s = (float)k, h = 0.5f * (float)(k - 1), inv = 1.f / (float)(k * k);
        for (int u = 0; u < k; u++)
          for (int w = 0; w < k; w++) {
            float dvv[4];
            ps_eval(c, a.psReg, s * X - h + (float)w, s * Y - h + (float)u, s, dvv);
            for (int t4 = 0; t4 < 4; t4++) dsum[t4] += dvv[t4] * inv;
          }
      } else {
        const float s = c.s1;
        if (!ps_far(a.psMain, s * X, s * Y)) ps_eval(c, a.psMain, s * X, s * Y, s, dsum);
      }
      const bool rot = d.type == F_POINTSOURCEROT;
      const int map[4] = {d.x0Index, d.x0Index + 1, d.paramOffset + (rot ? 1 : 0), rot ? d.paramOffset : -1};
      for (int t4 = 0; t4 < 4; t4++)
        if (map[t4] >= 0 && ss[map[t4]] >= 0) Zr[ss[map[t4]] * uStride + col] += q * dsum[t4];
    }
    qb[col] = q * (inReg ? a.psfSumOs : a.psfSum);
    cw[col] = cnt;
    dv[col] = dev;
    zero[col] = 0.f;
    if (jac) {  // Jacobian columns [b][param][pixel] and the deviates [b][pixel] after them
      float *jb = jac + (long)b * (nP + 1) * nPix;
      for (int j = 0; j < nP; j++) jb[(long)j * nPix + zi] = ss[j] >= 0 ? Zr[ss[j] * uStride + col] : qb[col];
      jb[(long)nP * nPix + zi] = dev;
    }
  }
  __syncthreads();
  const int Q = nP * (nP + 1) / 2 + nP + 1;
  float2 *out = part + (long)b * Q * a.partStride + blockIdx.x;
  if (a.count)
    jtwj_gram<true>(Zr, uStride, ss, qb, dv, zero, cw, nc, nP, red, out, a.partStride);
  else
    jtwj_gram<false>(Zr, uStride, ss, qb, dv, zero, cw, nc, nP, red, out, a.partStride);
}

// FP64 sums of the per-row partials: grid (quantity, parameter vector).
__global__ void __launch_bounds__(256) k_fast_jtwj_reduce(FastArgs a, const float2 *__restrict__ part, int nRows,
                                                         double *__restrict__ alpha, double *__restrict__ beta,
                                                         double *__restrict__ stat) {
  const int qi = blockIdx.x, b = blockIdx.y, nP = a.nParams;
  const int nPair = nP * (nP + 1) / 2, Q = nPair + nP + 1;
  const float2 *p = part + ((long)b * Q + qi) * a.partStride;
  double t = 0.0;
  for (int i = threadIdx.x; i < nRows; i += blockDim.x) t += (double)p[i].x + (double)p[i].y;
  t = block_sum_d(t);
  if (threadIdx.x != 0) return;
  if (qi < nPair) {
    int j = 0, r = qi;
    while (r >= nP - j) {
      r -= nP - j;
      j++;
    }
    const int k = j + r;
    alpha[((long)b * nP + j) * nP + k] = t;
    alpha[((long)b * nP + k) * nP + j] = t;
  } else if (qi < nPair + nP) {
    beta[(long)b * nP + (qi - nPair)] = t;
  } else {
    stat[b] = t;
  }
}

// ------------------------------------------------------------ launchers
static FFTPlan<float> plan32(const FFTLen &L, bool half) {
  FFTPlan<float> p;
  const FFTTable &t = half ? L.half : L.full;
  p.n = t.n;
  p.npass = t.npass;
  p.radix = pack_radix(t.radix, t.npass);
  p.tw = reinterpret_cast<const cplx<float> *>(t.tw32);
  return p;
}


// CTAs of the main window's statistic pass, and of the whole statistic (the
// region's block-average CTAs, one per replaced data row, take the slots after)
static int fast_stat_main_blocks(const FastGeom &g, const FastTune &t) {
  return (g.nDataRows + t.rowRpb - 1) / t.rowRpb;
}

int fast_stat_blocks(const FastGeom &g, const FastTune &t) {
  return fast_stat_main_blocks(g, t) + (g.hasRegion ? g.rRows : 0);
}

static WinDesc main_win(const FastGeom &g, void *spec) {
  WinDesc w{};
  w.cols = g.winCols;
  w.rows = g.winRows;
  w.isRegion = 0;
  w.xOrig = g.xOrig;
  w.yOrig = g.yOrig;
  w.specPitch = g.specPitch;
  w.specBatch = g.specBatch;
  w.spec = reinterpret_cast<cplx<float> *>(spec);
  return w;
}

static WinDesc region_win(const FastGeom &g, void *rspec) {
  WinDesc w{};
  w.cols = g.rWinCols;
  w.rows = g.rWinRows;
  w.isRegion = 1;
  w.x1 = g.rXBase;
  w.y1 = g.rYBase;
  w.offX = g.rWinOffX;
  w.offY = g.rWinOffY;
  w.scale = g.rScale;
  w.invScale = 1.f / (float)g.rScale;
  w.startOff = g.rStartOff;
  w.frac = g.rFrac;
  w.specPitch = g.rSpecPitch;
  w.specBatch = g.rSpecBatch;
  w.spec = reinterpret_cast<cplx<float> *>(rspec);
  return w;
}

int fast_grad_blocks(const FastGeom &g, const FastTune &t) {
  return (g.winRows + t.rowRpb - 1) / t.rowRpb;
}

int fast_reg_grad_blocks(const FastGeom &g, const FastTune &t) {
  if (!g.hasRegion) return 0;
  return (g.rWinRows + t.rowRpb - 1) / t.rowRpb;
}

template <typename K>
static void ensure_smem(K kern, size_t bytes) {
  (void)bytes;
  allow_max_smem((const void *)kern);
}

// Set-up and main-window subsample table: CTAs per (component, vector) chosen
// so that the grid is about one wave of 8 CTAs per SM, at most one warp per
// box pixel.
static cudaError_t launch_setup_subsample(const FastArgs &a, const WinDesc &mw, const WinDesc &rw, bool region,
                                          int nBatch, cudaStream_t st) {
  const int cap = std::max(1, 8 * 152 / std::max(a.nComp * nBatch, 1));
  const int n = std::max(1, std::min((a.boxMain * a.boxMain + 7) / 8, cap));
  return launch_pdl(k_fast_setup_subsample, dim3(n, a.nComp, nBatch), dim3(256), 0, st, a, mw, rw,
                    region ? 1 : 0);
}

// Set-up: one CTA per (component, vector).
static cudaError_t launch_setup(const FastArgs &a, const WinDesc &mw, const WinDesc &rw, bool region, int nBatch,
                                cudaStream_t st) {
  return launch_pdl(k_fast_setup, dim3(a.nComp, nBatch), dim3(256), 0, st, a, mw, rw, region ? 1 : 0);
}

// Subsample table of the main window: CTAs per (component, vector) chosen so
// that the grid is about one wave of 8 CTAs per SM, at most one warp per box
// pixel.
static cudaError_t launch_subsample(const FastArgs &a, const WinDesc &mw, int nBatch, cudaStream_t st) {
  const int cap = std::max(1, 8 * 152 / std::max(a.nComp * nBatch, 1));
  const int n = std::max(1, std::min((a.boxMain * a.boxMain + 7) / 8, cap));
  return launch_pdl(k_fast_subsample, dim3(n, a.nComp, nBatch), dim3(256), 0, st, a, mw);
}

// Subsample table of the oversampled region: the shared lattice (when the
// region's scale divides its subsample count), then the table.
static cudaError_t launch_region_sub(const FastArgs &a, const WinDesc &rw, int nBatch, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (a.lat) {
    const int pts = a.latSide * a.latSide;
    e = launch_pdl(k_fast_region_lattice, dim3((pts + 255) / 256, a.nComp, nBatch), dim3(256), 0, st, a, rw);
    if (e) return e;
  }
  // about two CTAs per SM: the region's pipeline runs beside the main
  // window's at a higher stream priority, and a full wave of these CTAs would
  // hold the SMs the main window's model pass is waiting for
  const int cap = std::max(1, 2 * 152 / std::max(a.nComp * nBatch, 1));
  const int n = std::max(1, std::min((a.boxReg * a.boxReg + 7) / 8, cap));
  return launch_pdl(k_fast_region_sub, dim3(n, a.nComp, nBatch), dim3(256), 0, st, a, rw);
}

static cudaError_t launch_eval(const FastArgs &a, const WinDesc &w, const FFTLen &L, int nBatch, int win,
                               const FastTune &tu, cudaStream_t st) {
  const int M = L.half.n;
  const int rpb = tu.rowRpb;
  const size_t sm = sizeof(CompF32) * kMaxComponents + sizeof(int) * 2 * kMaxComponents +
                    sizeof(cplx<float>) * 2 * rpb * (M + 1) + 16;
  ensure_smem(k_fast_eval_r2c, sm);
  dim3 grid((w.rows + rpb - 1) / rpb, nBatch);
  return launch_pdl(k_fast_eval_r2c, grid, dim3(tu.rowThreads), sm, st, a, w, plan32(L, true),
                    reinterpret_cast<const cplx<float> *>(L.twL32), rpb, win);
}

static cudaError_t launch_grad(const FastArgs &a, const WinDesc &w, const FFTLen &L, int nBatch, int blockBase,
                               int win, const FastTune &tu, cudaStream_t st, int doneTotal) {
  const int M = L.half.n;
  const int rpb = tu.rowRpb;
  const size_t sm = sizeof(CompF32) * kMaxComponents + sizeof(int) * 2 * kMaxComponents +
                    sizeof(cplx<float>) * 3 * rpb * (M + 1) + sizeof(ffloat) * (tu.rowThreads / 32) * a.nParams + 16;
  ensure_smem(k_fast_grad_rows, sm);
  dim3 grid((w.rows + rpb - 1) / rpb, nBatch);
  return launch_pdl(k_fast_grad_rows, grid, dim3(tu.rowThreads), sm, st, a, w, plan32(L, true),
                    reinterpret_cast<const cplx<float> *>(L.twL32), rpb, a.gradPart, blockBase, win, doneTotal);
}

static void record(cudaEvent_t ev, cudaStream_t st) {
  // while the stream is being captured the record must be External to become an
  // event-record node of the graph; outside capture that flag is not allowed
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cs);
  if (cs == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
  else
    cudaEventRecord(ev, st);
}

// called before a kernel of the given stage is launched
static void stage_begin(const FastPlan &p, const char *name, cudaStream_t st) {
  StageTimer *t = p.timer;
  if (t && t->only && strcmp(t->only, name) == 0) {
    record(t->ev[0], st);
    t->names[0] = "start";
  }
}

// called after the kernel of the stage has been launched
static void stage_end(const FastPlan &p, const char *name, cudaStream_t st) {
  StageTimer *t = p.timer;
  if (!t) return;
  if (t->only) {
    if (strcmp(t->only, name) == 0) {
      record(t->ev[1], st);
      t->names[1] = name;
      t->n = 2;
    }
    return;
  }
  if (t->n >= StageTimer::kMax) return;
  record(t->ev[t->n], st);
  t->names[t->n] = name;
  t->n++;
}

#define STAGE(name, stream, call)        \
  do {                                   \
    stage_begin(p, name, stream);        \
    cudaError_t e_ = (call);             \
    if (e_) return e_;                   \
    stage_end(p, name, stream);          \
  } while (0)

static cudaError_t launch_los_eval(const FastArgs &a, const WinDesc &w, int nBatch, LosStore ks, cudaStream_t st) {
  return launch_pdl(k_fast_los_eval, dim3(kLosCtas, nBatch), dim3(256), 0, st, a, w, ks);
}

static cudaError_t launch_los_grad(const FastArgs &a, const WinDesc &w, int nBatch, int blockBase, LosStore ks,
                                   cudaStream_t st, int doneTotal) {
  return launch_pdl(k_fast_los_grad, dim3(kLosCtas, nBatch), dim3(256), 0, st, a, w, a.gradPart, blockBase, ks,
                    doneTotal);
}

static cudaError_t launch_region_down(const FastPlan &p, const FastArgs &a, int nBatch, bool wantGrad,
                                      cudaStream_t st, int doneTotal) {
  const FastGeom &g = p.g;
  const int M = p.Rx->half.n;
  const size_t sm = sizeof(cplx<float>) * 3 * g.rScale * (M + 1);
  auto kern = a.nPs ? k_fast_region_down<true> : k_fast_region_down<false>;
  ensure_smem(kern, sm);
  return launch_pdl(kern, dim3(g.rRows, nBatch), dim3(line_threads(M * g.rScale / 2)), sm, st, a, g,
                    reinterpret_cast<cplx<float> *>(a.rspec), plan32(*p.Rx, true),
                    reinterpret_cast<const cplx<float> *>(p.Rx->twL32), (float *)nullptr, wantGrad ? 2 : 1,
                    fast_stat_main_blocks(g, p.tune), doneTotal);
}

static cudaError_t launch_stat(const FastPlan &p, const FastArgs &a, int nBatch, bool wantGrad, cudaStream_t st,
                               int doneTotal) {
  const FastGeom &g = p.g;
  const int M = p.Lx->half.n;
  const int rpb = p.tune.rowRpb;
  const size_t sm = sizeof(cplx<float>) * 3 * rpb * (M + 1);
  auto kern = a.nPs ? k_fast_stat_rows<true> : k_fast_stat_rows<false>;
  ensure_smem(kern, sm);
  dim3 grid((g.nDataRows + rpb - 1) / rpb, nBatch);
  return launch_pdl(kern, grid, dim3(p.tune.rowThreads), sm, st, a, g, plan32(*p.Lx, true),
                    reinterpret_cast<const cplx<float> *>(p.Lx->twL32), rpb, wantGrad ? 1 : 0, doneTotal);
}



// The whole statistic (+ gradient) evaluation.  With p.side set, the
// oversampled region's pipeline -- subsample table, model rows, convolution,
// block average with the region pixels' statistic, and with the gradient its
// adjoint -- runs on the side stream, forked after the set-up and joined at
// the end; the last CTA of either window's final pass adds up the partials.
cudaError_t fast_forward(const FastPlan &p, const FastArgs &a, int nBatch, bool wantGrad, cudaStream_t st) {
  const FastGeom &g = p.g;
  if (!a.done) return cudaErrorInvalidValue;  // the final reduction needs the completion counters
  if (p.timer) p.timer->n = 0;
  if (p.timer && !p.timer->only) stage_end(p, "start", st);
  const bool fork = g.hasRegion && p.side;
  cudaStream_t rs = fork ? p.side : st;
  const float scale = 1.f / ((float)p.Lx->L * (float)p.Ly->L);
  const float rscale = g.hasRegion ? 1.f / ((float)p.Rx->L * (float)p.Ry->L) : 0.f;
  const FastTune &tu = p.tune;
  const bool los = a.losVal != nullptr;
  const int nMain = fast_grad_blocks(g, tu), nReg = fast_reg_grad_blocks(g, tu);
  const int nLos = los ? kLosCtas * (g.hasRegion ? 2 : 1) : 0;
  const int nTot = nMain + nReg + nLos;
  const int nStat = fast_stat_blocks(g, tu);
  WinDesc mw = main_win(g, a.spec), rw = region_win(g, a.rspec);
  mw.losVal = a.losVal;
  mw.losRt = a.losRt;
  rw.losVal = a.rLosVal;
  rw.losRt = a.rLosRt;
  // kept partitions (only worth writing when the gradient pass follows)
  LosStore mks{wantGrad ? reinterpret_cast<float2 *>(a.losPan) : nullptr, a.losCnt, a.nLos};
  LosStore rks{wantGrad ? reinterpret_cast<float2 *>(a.rLosPan) : nullptr, a.rLosCnt, a.nLos};
  if (!mks.panels) mks.count = nullptr;
  if (!rks.panels) rks.count = nullptr;

  // one kernel for the set-up and the main window's table, unless the
  // region's pipeline waits to start after the set-up
  if (g.hasRegion) {
    STAGE("setup", st, launch_setup(a, mw, rw, true, nBatch, st));
  } else {
    STAGE("setup_subsample", st, launch_setup_subsample(a, mw, rw, false, nBatch, st));
  }
  if (fork) {
    cudaError_t e = cudaEventRecord(p.fork0, st);
    if (!e) e = cudaStreamWaitEvent(rs, p.fork0, 0);
    if (e) return e;
  }
  if (g.hasRegion) STAGE("region_subsample", rs, launch_region_sub(a, rw, nBatch, rs));
  if (g.hasRegion) STAGE("subsample", st, launch_subsample(a, mw, nBatch, st));
  if (g.hasRegion) {
    if (los) STAGE("region_los_eval", rs, launch_los_eval(a, rw, nBatch, rks, rs));
    STAGE("region_eval_r2c", rs, launch_eval(a, rw, *p.Rx, nBatch, 1, tu, rs));
    STAGE("region_cols_conv", rs,
          launch_cols32(a.rspec, g.rSpecPitch, g.rSpecBatch, p.Rx->L / 2 + 1, g.rWinRows, g.rSubRows, p.Hr,
                             p.hrPitch, *p.Ry, rscale, 1, nBatch, rs, tu.colCpb, 0, 1, nullptr, tu.colThreads));
    STAGE("region_down", rs, launch_region_down(p, a, nBatch, wantGrad, rs, wantGrad ? 0 : nStat));
    if (wantGrad) {
      STAGE("region_cols_adjoint", rs,
            launch_cols32(a.rspec, g.rSpecPitch, g.rSpecBatch, p.Rx->L / 2 + 1, g.rSubRows, g.rWinRows, p.Hr,
                          p.hrPitch, *p.Ry, rscale, 2, nBatch, rs, tu.colCpb, 0, 1, nullptr, tu.colThreads));
      STAGE("region_grad_rows", rs, launch_grad(a, rw, *p.Rx, nBatch, nMain, 1, tu, rs, nTot));
      if (los) STAGE("region_los_grad", rs, launch_los_grad(a, rw, nBatch, nMain + nReg + kLosCtas, rks, rs, nTot));
    }
  }
  if (los) STAGE("los_eval", st, launch_los_eval(a, mw, nBatch, mks, st));
  STAGE("eval_r2c", st, launch_eval(a, mw, *p.Lx, nBatch, 0, tu, st));
  STAGE("cols_conv", st,
        launch_cols32(a.spec, g.specPitch, g.specBatch, p.Lx->L / 2 + 1, g.winRows, g.nDataRows, p.H, p.hPitch,
                           *p.Ly, scale, 1, nBatch, st, tu.colCpb, p.hBatch, 1, p.hMap, tu.colThreads));
  // without the gradient the statistic passes are the last ones: the final
  // CTA per vector adds the partials up; with it, the gradient passes' last CTA does
  STAGE("stat_rows", st, launch_stat(p, a, nBatch, wantGrad, st, wantGrad ? 0 : nStat));
  if (!wantGrad) {
    if (fork) {
      cudaError_t e = cudaEventRecord(p.join0, rs);
      if (!e) e = cudaStreamWaitEvent(st, p.join0, 0);
      if (e) return e;
    }
    return cudaSuccess;
  }
  STAGE("cols_adjoint", st,
        launch_cols32(a.spec, g.specPitch, g.specBatch, p.Lx->L / 2 + 1, g.nDataRows, g.winRows, p.H, p.hPitch,
                           *p.Ly, scale, 2, nBatch, st, tu.colCpb, p.hBatch, 1, p.hMap, tu.colThreads));
  STAGE("grad_rows", st, launch_grad(a, mw, *p.Lx, nBatch, 0, 0, tu, st, nTot));
  if (los) STAGE("los_grad", st, launch_los_grad(a, mw, nBatch, nMain + nReg, mks, st, nTot));
  if (fork) {
    cudaError_t e = cudaEventRecord(p.join1, rs);
    if (!e) e = cudaStreamWaitEvent(st, p.join1, 0);
    if (e) return e;
  }
  return cudaSuccess;
}

// ----------------------------------------------------- JtWJ (forward mode)
static size_t deriv_smem(int M, int nD) {
  return sizeof(CompF32) * kMaxComponents + sizeof(int) * (3 * kMaxComponents + kMaxParams) +
         sizeof(cplx<float>) * 2 * (size_t)nD * (M + 1) + 16;
}

// The two FFT buffers, plus room for the per-pixel vectors and chunk sums of
// jtwj_gram when they do not fit in the buffer the transform leaves free.
static size_t jtwj_rows_smem(int M, int nD, int nP, int nCols, int threads) {
  const long aux = jtwj_aux_floats(nP, nCols, threads);
  const long spare = 2L * nD * (M + 1);
  return sizeof(int) * kMaxParams + sizeof(cplx<float>) * 2 * (size_t)nD * (M + 1) +
         (aux <= spare ? 0 : sizeof(float) * (size_t)aux) + 16;
}

static constexpr int kJtwjThreads = 512;

size_t fast_jtwj_smem(const FastPlan &p, int nD, int nP) {
  size_t s = deriv_smem(p.Lx->half.n, nD);
  s = std::max(s, jtwj_rows_smem(p.Lx->half.n, nD, nP, p.g.nDataCols, kJtwjThreads));
  if (p.g.hasRegion) s = std::max(s, deriv_smem(p.Rx->half.n, nD));
  return s;
}

static cudaError_t launch_deriv(const FastArgs &a, const WinDesc &w, const FFTLen &L, int nBatch, int win,
                                const JtwjArgs &J, cudaStream_t st) {
  const int M = L.half.n;
  const size_t sm = deriv_smem(M, J.nD);
  k_fast_deriv_r2c<<<dim3(w.rows, nBatch), kJtwjThreads, sm, st>>>(
      a, w, plan32(L, true), reinterpret_cast<const cplx<float> *>(L.twL32), J.slot, J.nD, win);
  return cudaGetLastError();
}

// Statistic, JtJ and Jt dev of the deviates for nBatch parameter vectors:
// the forward pass (which leaves the FP32 model image in a.modelOut), the
// derivative images of every non-background parameter convolved with the PSF
// (region derivatives through the oversampled pipeline and the block
// average), then the per-row products and their FP64 sums.
cudaError_t fast_jtwj(const FastPlan &p, const FastArgs &a, const JtwjArgs &J, int nBatch, cudaStream_t st) {
  const FastGeom &g = p.g;
  cudaError_t e = fast_forward(p, a, nBatch, false, st);
  if (e) return e;
  const int nD = J.nD, nB = nBatch * nD;
  const FastTune &tu = p.tune;
  if (nD > 0) {
    if (g.hasRegion) {
      const float rscale = 1.f / ((float)p.Rx->L * (float)p.Ry->L);
      STAGE("jtwj_region_deriv_r2c", st, launch_deriv(a, region_win(g, J.drspec), *p.Rx, nBatch, 1, J, st));
      STAGE("jtwj_region_cols", st,
            launch_cols32(J.drspec, g.rSpecPitch, g.rSpecBatch, p.Rx->L / 2 + 1, g.rWinRows, g.rSubRows, p.Hr,
                               p.hrPitch, *p.Ry, rscale, 1, nB, st, tu.colCpb, 0, 1, nullptr, tu.colThreads));
      const int M = p.Rx->half.n;
      const size_t sm = sizeof(cplx<float>) * 3 * g.rScale * (M + 1);
      stage_begin(p, "jtwj_region_down", st);
      k_fast_region_down<false><<<dim3(g.rRows, nB), line_threads(M * g.rScale / 2), sm, st>>>(
          a, g, reinterpret_cast<cplx<float> *>(J.drspec), plan32(*p.Rx, true),
          reinterpret_cast<const cplx<float> *>(p.Rx->twL32), J.regDeriv, 0, 0, 0);
      if ((e = cudaGetLastError())) return e;
      stage_end(p, "jtwj_region_down", st);
    }
    const float scale = 1.f / ((float)p.Lx->L * (float)p.Ly->L);
    STAGE("jtwj_deriv_r2c", st, launch_deriv(a, main_win(g, J.dspec), *p.Lx, nBatch, 0, J, st));
    STAGE("jtwj_cols", st,
          launch_cols32(J.dspec, g.specPitch, g.specBatch, p.Lx->L / 2 + 1, g.winRows, g.nDataRows, p.H,
                             p.hPitch, *p.Ly, scale, 1, nB, st, tu.colCpb, p.hBatch, nD, p.hMap, tu.colThreads));
  }
  const int M = p.Lx->half.n;
  const size_t sm = jtwj_rows_smem(M, nD, a.nParams, g.nDataCols, kJtwjThreads);
  stage_begin(p, "jtwj_rows", st);
  auto jrows = a.nPs ? k_fast_jtwj_rows<true> : k_fast_jtwj_rows<false>;
  jrows<<<dim3(g.nDataRows, nBatch), kJtwjThreads, sm, st>>>(
      a, g, plan32(*p.Lx, true), reinterpret_cast<const cplx<float> *>(p.Lx->twL32),
      reinterpret_cast<const cplx<float> *>(J.dspec), J.regDeriv, J.slot, nD, J.part, J.jac);
  if ((e = cudaGetLastError())) return e;
  stage_end(p, "jtwj_rows", st);
  const int nP = a.nParams, Q = nP * (nP + 1) / 2 + nP + 1;
  stage_begin(p, "jtwj_reduce", st);
  k_fast_jtwj_reduce<<<dim3(Q, nBatch), 256, 0, st>>>(a, J.part, g.nDataRows, J.alpha, J.beta, J.stat);
  if ((e = cudaGetLastError())) return e;
  stage_end(p, "jtwj_reduce", st);
  return cudaSuccess;
}

// ======================================================= ragged cutout sets
// The J^T W J evaluation of a ragged cutout set (one model, many cutouts of
// different sizes; see RagEntry): the same stages as fast_forward + fast_jtwj
// for a single image, each one launch over all active cutouts.  Per-evaluation
// state (parameters, component records, subsample tables, background levels,
// outputs) is indexed by the slot k of the active list; per-cutout data
// (images, PSF spectra, spectra, model images, row partials) by its entry.

__device__ __forceinline__ WinDesc rag_win(const RagEntry &E, cplx<float> *spec) {
  WinDesc w{};
  w.cols = E.winCols;
  w.rows = E.winRows;
  w.isRegion = 0;
  w.xOrig = E.xOrig;
  w.yOrig = E.yOrig;
  w.specPitch = E.pitch;
  w.specBatch = E.specSize;
  w.spec = spec;
  return w;
}

// Set-up of component c for slot k, then its subsampled pixels (one warp per
// box pixel, grid-stride over the gridDim.x CTAs of the slot and component).
__global__ void __launch_bounds__(256) k_rag_subsample(FastArgs a, RagArgs r) {
  pdl_wait();
  const int k = blockIdx.z, c = blockIdx.y;
  if (blockIdx.x != 0 && !(a.desc[c].subsample && subsampling_type(a.desc[c].type))) return;
  __shared__ CompF32 rec;
  setup_component(a, c, k, rec, blockIdx.x == 0 && c == 0);
  const CompF32 cc = rec;
  if (blockIdx.x == 0 && threadIdx.x == 0) a.comps[k * a.nComp + c] = cc;
  if (!cc.subsample || !subsampling_type(cc.type)) return;
  const RagEntry &E = r.ent[r.act[k]];
  const WinDesc w = rag_win(E, nullptr);
  const int side = a.boxMain;
  int col0, row0;
  box_origin(w, cc, side, col0, row0);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int *o = a.subBox + ((long)k * a.nComp + c) * 4;
    o[0] = col0;
    o[1] = row0;
  }
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const FastDiv bySide(side);
  for (int p = blockIdx.x * nw + (threadIdx.x >> 5); p < side * side; p += gridDim.x * nw) {
    const int pr = bySide.div(p);
    const int row = row0 + pr, col = col0 + (p - pr * side);
    if (row < 0 || row >= w.rows || col < 0 || col >= w.cols) continue;
    float dx, dy;
    win_offsets(w, cc, row, col, dx, dy);
    const Geo g = geo32(cc, dx, dy);
    const int ns = sub_count(cc, g);
    if (ns <= 1) continue;
    const float d = 1.f / ns;
    const float xs = dx - 0.5f + 0.5f * d, ys = dy - 0.5f + 0.5f * d;
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    switch (cc.type) {
      case F_SERSIC: subsample_sum<F_SERSIC>(cc, ns, xs, ys, d, lane, acc); break;
      case F_EXP: subsample_sum<F_EXP>(cc, ns, xs, ys, d, lane, acc); break;
      case F_MOFFAT: subsample_sum<F_MOFFAT>(cc, ns, xs, ys, d, lane, acc); break;
      default: subsample_sum<F_GAUSS>(cc, ns, xs, ys, d, lane, acc); break;
    }
#pragma unroll
    for (int q = 0; q < 8; q++) acc[q] = warp_sum(acc[q]);
    if (lane == 0) {
      float *dst = a.subTab + sub_base(a, k, c, 0) + (long)p * 8;
      const float dd = d * d;
#pragma unroll
      for (int q = 0; q < 8; q++) dst[q] = acc[q] * dd;
    }
  }
}

// One window row of one cutout per CTA: evaluated model row, row r2c.
__global__ void __launch_bounds__(512) k_rag_eval_r2c(FastArgs a, RagArgs r) {
  extern __shared__ __align__(16) unsigned char smem[];
  pdl_wait();
  const int t = blockIdx.x;
  const int k = rag_slot(r.start, r.K, t);
  const RagEntry &E = r.ent[r.act[k]];
  const int row = t - r.start[k];
  const int M = E.rowPlan.n, ls = M + 1;
  CompF32 *sc = reinterpret_cast<CompF32 *>(smem);
  int *boxes = reinterpret_cast<int *>(sc + kMaxComponents);
  cplx<float> *bufA = reinterpret_cast<cplx<float> *>(boxes + 2 * kMaxComponents);
  cplx<float> *bufB = bufA + ls;
  const int nC = a.nComp;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) {
    sc[i] = a.comps[k * nC + i];
    const int *o = a.subBox + ((long)k * nC + i) * 4;
    boxes[2 * i] = o[0];
    boxes[2 * i + 1] = o[1];
  }
  for (int i = threadIdx.x; i < M; i += blockDim.x) bufA[i] = {0.f, 0.f};
  __syncthreads();
  const WinDesc w = rag_win(E, r.spec + E.specOff);
  const FastDiv byM(M);
  for (int c = 0; c < nC; c++) {
    const CompF32 cc = sc[c];
    if (!in_rows(cc.type)) continue;
    const float *tab = a.subTab + sub_base(a, k, c, 0);
    const int bc0 = boxes[2 * c], br0 = boxes[2 * c + 1], side = a.boxMain;
    const bool box = rows_meet_box(cc, row, 1, br0, side);
    switch (cc.type) {
      case F_SERSIC: eval_pixels_rt<F_SERSIC>(false, box, cc, w, row, 1, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_EXP: eval_pixels_rt<F_EXP>(false, box, cc, w, row, 1, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_GRING: eval_pixels_rt<F_GRING>(false, box, cc, w, row, 1, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_MOFFAT: eval_pixels_rt<F_MOFFAT>(false, box, cc, w, row, 1, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_GAUSS: eval_pixels_rt<F_GAUSS>(false, box, cc, w, row, 1, M, ls, byM, bufA, tab, side, bc0, br0); break;
      case F_TILTEDSKY: eval_pixels_rt<F_TILTEDSKY>(false, box, cc, w, row, 1, M, ls, byM, bufA, tab, side, bc0, br0); break;
      default: break;
    }
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, E.rowPlan, 1, ls, 1, -1, false);
  pdl_trigger();
  cplx<float> *out = w.spec + (long)row * E.pitch;
  for (int kk = threadIdx.x; kk <= M; kk += blockDim.x) out[kk] = r2c_post(Z, kk, M, E.twL);
}

// One data row of one cutout per CTA: inverse row FFT of the convolved
// spectrum, the FP32 model row (plus the constant background) to r.model.
__global__ void __launch_bounds__(512) k_rag_model_rows(FastArgs a, RagArgs r) {
  extern __shared__ __align__(16) unsigned char smem[];
  pdl_wait();
  const int t = blockIdx.x;
  const int k = rag_slot(r.start, r.K, t);
  const RagEntry &E = r.ent[r.act[k]];
  const int row = t - r.start[k];
  const int M = E.rowPlan.n, ls = M + 1;
  cplx<float> *bufX = reinterpret_cast<cplx<float> *>(smem);
  cplx<float> *bufA = bufX + ls;
  cplx<float> *bufB = bufA + ls;
  const cplx<float> *in = r.spec + E.specOff + (long)row * E.pitch;
  for (int kk = threadIdx.x; kk <= M; kk += blockDim.x) bufX[kk] = in[kk];
  __syncthreads();
  for (int kk = threadIdx.x; kk < M; kk += blockDim.x) bufA[kk] = c2r_pre(bufX, kk, M, E.twL);
  __syncthreads();
  const cplx<float> *Z = block_fft(bufA, bufB, E.rowPlan, 1, ls, 1, +1, false);
  pdl_trigger();
  const float *zr = reinterpret_cast<const float *>(Z);
  const float bg = a.bgLevel[2 * k];
  float *m = r.model + E.dataOff + (long)row * E.nDataCols;
  for (int col = threadIdx.x; col < E.nDataCols; col += blockDim.x) m[col] = zr[col] + bg;
}

// One window row of one cutout per CTA: the nD derivative rows (typed pixel
// passes), their row FFTs, to derivative spectrum j of the cutout.
__global__ void __launch_bounds__(512) k_rag_deriv_r2c(FastArgs a, RagArgs r, const int *__restrict__ slot, int nD) {
  extern __shared__ __align__(16) unsigned char smem[];
  pdl_wait();
  const int t = blockIdx.x;
  const int k = rag_slot(r.start, r.K, t);
  const RagEntry &E = r.ent[r.act[k]];
  const int row = t - r.start[k];
  const int M = E.rowPlan.n, ls = M + 1;
  CompF32 *sc = reinterpret_cast<CompF32 *>(smem);
  int *boxes = reinterpret_cast<int *>(sc + kMaxComponents);
  int *npar = boxes + 2 * kMaxComponents;
  int *ss = npar + kMaxComponents;
  cplx<float> *bufA = reinterpret_cast<cplx<float> *>(ss + kMaxParams);
  cplx<float> *bufB = bufA + nD * ls;
  const int nC = a.nComp;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) {
    sc[i] = a.comps[k * nC + i];
    const int *o = a.subBox + ((long)k * nC + i) * 4;
    boxes[2 * i] = o[0];
    boxes[2 * i + 1] = o[1];
    npar[i] = a.desc[i].nParams;
  }
  for (int i = threadIdx.x; i < a.nParams; i += blockDim.x) ss[i] = slot[i];
  for (int i = threadIdx.x; i < nD * ls; i += blockDim.x) bufA[i] = {0.f, 0.f};
  __syncthreads();
  float *lines = reinterpret_cast<float *>(bufA);
  const WinDesc w = rag_win(E, nullptr);
  for (int c = 0; c < nC; c++) {
    const CompF32 cc = sc[c];
    if (!in_rows(cc.type)) continue;
    int sl[7];
    sl[0] = ss[cc.x0Index];
    sl[1] = ss[cc.x0Index + 1];
#pragma unroll
    for (int q = 0; q < 5; q++) sl[2 + q] = q < npar[c] ? ss[cc.paramOffset + q] : -1;
    const float *tab = a.subTab + sub_base(a, k, c, 0);
    const int bc0 = boxes[2 * c], br0 = boxes[2 * c + 1], side = a.boxMain;
    const bool box = rows_meet_box(cc, row, 1, br0, side);
    switch (cc.type) {
      case F_SERSIC: deriv_pixels_rt<F_SERSIC>(false, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_EXP: deriv_pixels_rt<F_EXP>(false, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_GRING: deriv_pixels_rt<F_GRING>(false, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_MOFFAT: deriv_pixels_rt<F_MOFFAT>(false, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_GAUSS: deriv_pixels_rt<F_GAUSS>(false, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      case F_TILTEDSKY: deriv_pixels_rt<F_TILTEDSKY>(false, box, cc, w, row, sl, lines, ls, tab, side, bc0, br0); break;
      default: break;
    }
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, E.rowPlan, nD, ls, 1, -1, false);
  pdl_trigger();
  cplx<float> *out = r.spec + (long)nD * E.specOff + (long)row * E.pitch;
  const FastDiv byM1(M + 1);
  for (int idx = threadIdx.x; idx < nD * (M + 1); idx += blockDim.x) {
    const int j = byM1.div(idx), kk = idx - j * (M + 1);
    out[(long)j * E.specSize + kk] = r2c_post(Z + j * ls, kk, M, E.twL);
  }
}

// One data row of one cutout per CTA: inverse FFTs of the nD convolved
// derivative rows, the Jacobian rows u_j = q dM/dtheta_j of the deviates and
// the row's FP32 partial sums of alpha_jk (j <= k), beta_j and S.
__global__ void __launch_bounds__(512) k_rag_jtwj_rows(FastArgs a, RagArgs r, const int *__restrict__ slot, int nD) {
  extern __shared__ __align__(16) unsigned char smem[];
  pdl_wait();
  const int t = blockIdx.x;
  const int k = rag_slot(r.start, r.K, t);
  const RagEntry &E = r.ent[r.act[k]];
  const int row = t - r.start[k];
  const int M = E.rowPlan.n, ls = M + 1, nP = a.nParams, nc = E.nDataCols;
  int *ss = reinterpret_cast<int *>(smem);
  cplx<float> *bufA = reinterpret_cast<cplx<float> *>(ss + kMaxParams);
  cplx<float> *bufB = bufA + nD * ls;
  for (int i = threadIdx.x; i < nP; i += blockDim.x) ss[i] = slot[i];
  const cplx<float> *src = r.spec + (long)nD * E.specOff + (long)row * E.pitch;
  const FastDiv byM(M);
  for (int idx = threadIdx.x; idx < nD * M; idx += blockDim.x) {
    const int j = byM.div(idx), kk = idx - j * M;
    bufA[j * ls + kk] = c2r_pre(src + (long)j * E.specSize, kk, M, E.twL);
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, E.rowPlan, nD, ls, 1, +1, false);
  // Jacobian rows in place over the real rows (row j at Zr + 2 j ls); the
  // per-pixel vectors in the free FFT buffer when they fit, else after bufB
  float *Zr = reinterpret_cast<float *>(Z);
  const long uStride = 2L * ls;
  float *aux = (jtwj_aux_floats(nP, nc, blockDim.x) <= 2 * nD * ls)
                   ? reinterpret_cast<float *>(Z == bufA ? bufB : bufA)
                   : reinterpret_cast<float *>(bufB + nD * ls);
  float *qb = aux, *dv = qb + 2 * nc, *zero = dv + nc, *red = zero + nc;
  for (int col = threadIdx.x; col < nc; col += blockDim.x) {
    const long z = E.dataOff + (long)row * nc + col;
    const float m = r.model[z];
    float dev, q;
    deviate_slope(a, z, m, dev, q);
    for (int j = 0; j < nD; j++) Zr[j * uStride + col] *= q;
    qb[col] = q * a.psfSum;
    dv[col] = dev;
    zero[col] = 0.f;
  }
  __syncthreads();
  pdl_trigger();
  jtwj_gram<false>(Zr, uStride, ss, qb, dv, zero, nullptr, nc, nP, red, r.part + (long)E.rowOff + row,
                   r.totalRows);
}

// FP64 sums over each cutout's row partials: grid (quantity, slot).
__global__ void __launch_bounds__(256) k_rag_jtwj_reduce(FastArgs a, RagArgs r, double *__restrict__ alpha,
                                                        double *__restrict__ beta, double *__restrict__ stat) {
  pdl_wait();
  const int qi = blockIdx.x, k = blockIdx.y, nP = a.nParams;
  const int nPair = nP * (nP + 1) / 2;
  const RagEntry &E = r.ent[r.act[k]];
  const float2 *p = r.part + (long)qi * r.totalRows + E.rowOff;
  double t = 0.0;
  for (int i = threadIdx.x; i < E.nDataRows; i += blockDim.x) t += (double)p[i].x + (double)p[i].y;
  t = block_sum_d(t);
  if (threadIdx.x != 0) return;
  if (qi < nPair) {
    int j = 0, rr = qi;
    while (rr >= nP - j) {
      rr -= nP - j;
      j++;
    }
    const int kk = j + rr;
    alpha[((long)k * nP + j) * nP + kk] = t;
    alpha[((long)k * nP + kk) * nP + j] = t;
  } else if (qi < nPair + nP) {
    beta[(long)k * nP + (qi - nPair)] = t;
  } else {
    stat[k] = t;
  }
}

static size_t rag_eval_smem(int maxM) {
  return sizeof(CompF32) * kMaxComponents + sizeof(int) * 2 * kMaxComponents + sizeof(cplx<float>) * 2 * (maxM + 1) +
         16;
}

constexpr int kRagRowThreads = 128;
constexpr int kRagJtwjThreads = 256;

size_t rag_jtwj_smem(int maxM, int nD, int nP, int maxCols) {
  const size_t deriv = sizeof(CompF32) * kMaxComponents + sizeof(int) * (3 * kMaxComponents + kMaxParams) +
                       sizeof(cplx<float>) * 2 * (size_t)nD * (maxM + 1) + 16;
  const size_t rows = sizeof(int) * kMaxParams + sizeof(cplx<float>) * 2 * (size_t)nD * (maxM + 1) +
                      sizeof(float) * (size_t)jtwj_aux_floats(nP, maxCols, kRagJtwjThreads) + 16;
  return std::max(deriv, rows);
}

// The whole ragged J^T W J evaluation: forward model (set-up + subsample,
// window rows + row FFT, column pass x PSF, inverse rows -> model images),
// derivative images (window rows, column pass x PSF), the per-row products
// and their FP64 sums per cutout.  r.spec holds the forward spectra, dspec the
// derivative spectra; starts/totals are the slots' prefix sums and totals per
// kind of work.
cudaError_t rag_jtwj(const FastArgs &a, RagArgs r, cplx<float> *dspec, const int *const starts[kRagWorkKinds],
                     const int totals[kRagWorkKinds], const int *slot, int nD, int maxM, int maxLy, int maxCols,
                     double *alpha, double *beta, double *stat, cudaStream_t st) {
  const int K = r.K;
  if (K <= 0) return cudaSuccess;
  cudaError_t e;
  // set-up + subsample tables: about 8 CTAs per SM over all slots and components
  const int cap = std::max(1, 8 * 152 / std::max(a.nComp * K, 1));
  const int nSub = std::max(1, std::min((a.boxMain * a.boxMain + 7) / 8, cap));
  if ((e = launch_pdl(k_rag_subsample, dim3(nSub, a.nComp, K), dim3(256), 0, st, a, r))) return e;
  r.start = starts[kRagWinRows];
  allow_max_smem((const void *)k_rag_eval_r2c);
  if ((e = launch_pdl(k_rag_eval_r2c, dim3(totals[kRagWinRows]), dim3(kRagRowThreads), rag_eval_smem(maxM), st, a,
                      r)))
    return e;
  r.start = starts[kRagCols];
  r.lines = 1;
  if ((e = launch_rag_cols(r, totals[kRagCols], maxLy, st))) return e;
  r.start = starts[kRagDataRows];
  allow_max_smem((const void *)k_rag_model_rows);
  if ((e = launch_pdl(k_rag_model_rows, dim3(totals[kRagDataRows]), dim3(kRagRowThreads),
                      sizeof(cplx<float>) * 3 * (maxM + 1), st, a, r)))
    return e;
  const size_t smJ = rag_jtwj_smem(maxM, nD, a.nParams, maxCols);
  RagArgs rd = r;
  rd.spec = dspec;
  if (nD > 0) {
    rd.start = starts[kRagWinRows];
    allow_max_smem((const void *)k_rag_deriv_r2c);
    if ((e = launch_pdl(k_rag_deriv_r2c, dim3(totals[kRagWinRows]), dim3(kRagJtwjThreads), smJ, st, a, rd, slot,
                        nD)))
      return e;
    rd.start = starts[kRagDerivCols];
    rd.lines = nD;
    if ((e = launch_rag_cols(rd, totals[kRagDerivCols], maxLy, st))) return e;
  }
  rd.start = starts[kRagDataRows];
  allow_max_smem((const void *)k_rag_jtwj_rows);
  if ((e = launch_pdl(k_rag_jtwj_rows, dim3(totals[kRagDataRows]), dim3(kRagJtwjThreads), smJ, st, a, rd, slot, nD)))
    return e;
  const int nP = a.nParams, Q = nP * (nP + 1) / 2 + nP + 1;
  return launch_pdl(k_rag_jtwj_reduce, dim3(Q, K), dim3(256), 0, st, a, rd, alpha, beta, stat);
}

void fast_prepare_kernels() {
  cols32_prepare_kernels();
  allow_max_smem((const void *)k_fast_eval_r2c);
  allow_max_smem((const void *)k_fast_grad_rows);
  allow_max_smem((const void *)k_fast_stat_rows<false>);
  allow_max_smem((const void *)k_fast_stat_rows<true>);
  allow_max_smem((const void *)k_fast_region_down<false>);
  allow_max_smem((const void *)k_fast_region_down<true>);
  allow_max_smem((const void *)k_fast_deriv_r2c);
  allow_max_smem((const void *)k_fast_jtwj_rows<false>);
  allow_max_smem((const void *)k_fast_jtwj_rows<true>);
}

}  // namespace imfit
