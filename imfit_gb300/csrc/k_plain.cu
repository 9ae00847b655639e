// k_plain.cu -- the plain FP64 path: the drop-in for ModelObject's
// CreateModelImage / ComputeDeviates / GetFitStatistic.
//
// Compiled with --fmad=false: every expression is evaluated in the same order
// and with the same rounding as the reference's (non-FMA) x86 build, so the
// per-pixel model matches ModelObject::CreateModelImage to a few ulp (the
// transcendental functions are CUDA's, not glibc's).
#include "kernels.h"
#include "stat_common.cuh"

namespace imfit {

// Coordinates of model pixel (i, j): IRAF pixel centres on the main grid,
// subpixel centres on a region grid.
__device__ __forceinline__ void pixel_xy64(const Grid64 &g, long i, long j, double &x, double &y) {
  if (!g.isRegion) {
    y = (double)(i - g.pr + 1);
    x = (double)(j - g.pc + 1);
  } else {
    y = g.y1 + g.off + (i - g.pr) * g.frac;
    x = g.x1 + g.off + (j - g.pc) * g.frac;
  }
}

// Subsample count at (x, y), with comp_value64_2d's expressions.
__device__ __forceinline__ int n_subsamples_at64(const CompF64 &c, double x, double y) {
  const double x_diff = x - c.x0, y_diff = y - c.y0;
  const double xp = x_diff * c.cosPA + y_diff * c.sinPA;
  const double yps = (-x_diff * c.sinPA + y_diff * c.cosPA) / c.q;
  return n_subsamples64(c, sqrt(xp * xp + yps * yps));
}

// Box of 2 subHalf x 2 subHalf pixels around component c's centre: every
// pixel within radius 10 of it (the only ones the subsampling rules touch)
// lies inside.  Origin (j0, i0).
__device__ __forceinline__ void sub_box64(const Grid64 &g, const CompF64 &c, long &j0, long &i0) {
  double jc, ic;
  if (!g.isRegion) {
    jc = c.x0 + g.pc - 1;
    ic = c.y0 + g.pr - 1;
  } else {
    jc = (c.x0 - g.x1 - g.off) / g.frac + g.pc;
    ic = (c.y0 - g.y1 - g.off) / g.frac + g.pr;
  }
  j0 = (long)floor(jc) - g.subHalf + 1;
  i0 = (long)floor(ic) - g.subHalf + 1;
}

size_t sub_table_size(const Grid64 &g, int nComp) {
  const long S = 2L * g.subHalf;
  return (size_t)nComp * S * S;
}

// One warp per (component, box pixel) that needs subsampling: the ns x ns
// subsamples of comp_value64_2d (same expressions, same (ii, jj) order within
// each lane's share) split over the lanes, the 32 partial sums added by a
// fixed shuffle tree.  The reference sums them in one sequence; the two orders
// differ by FP64 rounding only (~1e-16 relative), while one thread summing up
// to 10^4 subsamples (a Gaussian with sigma ~1: ns = 40 per axis) would set the
// whole image's latency.
__global__ void __launch_bounds__(256) k_sub64(const CompF64 *__restrict__ comps, Grid64 g) {
  const CompF64 cc = comps[blockIdx.y];
  if (!cc.subsample) return;
  const long S = 2L * g.subHalf;
  const long p = blockIdx.x * (long)(blockDim.x >> 5) + (threadIdx.x >> 5);
  if (p >= S * S) return;
  long j0, i0;
  sub_box64(g, cc, j0, i0);
  const long i = i0 + p / S, j = j0 + p % S;
  if (i < 0 || i >= g.nRows || j < 0 || j >= g.nCols) return;
  double x, y;
  pixel_xy64(g, i, j, x, y);
  const int ns = n_subsamples_at64(cc, x, y);
  if (ns <= 1) return;
  const int lane = threadIdx.x & 31;
  const double d = 1.0 / ns;
  const double xs0 = x - 0.5 + 0.5 * d;
  const double ys0 = y - 0.5 + 0.5 * d;
  double sum = 0.0;
  for (int t = lane; t < ns * ns; t += 32) {
    const int ii = t / ns, jj = t - ii * ns;
    const double xi = xs0 + ii * d;
    const double yi = ys0 + jj * d;
    const double x_diff = xi - cc.x0, y_diff = yi - cc.y0;
    const double xp = x_diff * cc.cosPA + y_diff * cc.sinPA;
    const double yps = (-x_diff * cc.sinPA + y_diff * cc.cosPA) / cc.q;
    sum += radial64(cc, sqrt(xp * xp + yps * yps));
  }
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) g.sub[(long)blockIdx.y * S * S + p] = sum / (ns * ns);
}

// CreateModelImage pixel loop: core/model_object.cpp:1144-1175 (main grid),
// OversampledRegion::ComputeRegionAndDownsample core/oversampled_region.cpp:301-327
// (region grid).  One thread per model pixel; Kahan sum over components;
// subsampled pixels from k_sub64's table.
__global__ void __launch_bounds__(256) k_eval64(const CompF64 *__restrict__ comps, int nComp,
                                                double *__restrict__ model, long pitch, Grid64 g,
                                                const double *__restrict__ los) {
  __shared__ CompF64 sc[kMaxComponents];
  for (int i = threadIdx.x; i < nComp; i += blockDim.x) sc[i] = comps[i];
  __syncthreads();
  const long n = (long)g.nCols * g.nRows;
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long j = k % g.nCols, i = k / g.nCols;
  double x, y;
  pixel_xy64(g, i, j, x, y);
  const long S = 2L * g.subHalf;
  double s = 0.0, err = 0.0;
  for (int c = 0; c < nComp; c++) {
    const int t = sc[c].type;
    if (is_point_source(t)) continue;  // added after the convolution
    double v;
    if (t == F_EXPDISK3D || t == F_FERRERS3D) {
      v = los[(long)sc[c].pad0 * n + k];
    } else if (!g.sub || t == F_FLATSKY || t == F_TILTEDSKY) {
      v = comp_value64_2d(sc[c], x, y);
    } else {
      // comp_value64_2d with the subsampled pixels read from the table
      const CompF64 &cc = sc[c];
      const double x_diff = x - cc.x0, y_diff = y - cc.y0;
      const double xp = x_diff * cc.cosPA + y_diff * cc.sinPA;
      const double yps = (-x_diff * cc.sinPA + y_diff * cc.cosPA) / cc.q;
      const double r = sqrt(xp * xp + yps * yps);
      if (n_subsamples64(cc, r) > 1) {
        long j0, i0;
        sub_box64(g, cc, j0, i0);
        const long bi = i - i0, bj = j - j0;
        v = (bi >= 0 && bi < S && bj >= 0 && bj < S) ? g.sub[(long)c * S * S + bi * S + bj]
                                                     : comp_value64_2d(cc, x, y);
      } else {
        v = radial64(cc, r);
      }
    }
    const double adj = v - err;
    const double tmp = s + adj;
    err = (tmp - s) - adj;
    s = tmp;
  }
  model[i * pitch + j] = s;
}

cudaError_t launch_eval64(const CompF64 *comps, int nComp, double *model, long pitch, Grid64 g,
                          const double *los, cudaStream_t st) {
  const long n = (long)g.nCols * g.nRows;
  if (n == 0) return cudaSuccess;
  if (g.sub) {
    const long S = 2L * g.subHalf;
    k_sub64<<<dim3((unsigned)((S * S + 7) / 8), (unsigned)nComp), 256, 0, st>>>(comps, g);
  }
  k_eval64<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(comps, nComp, model, pitch, g, los);
  return cudaGetLastError();
}

// Point sources after the convolution: core/model_object.cpp:1183-1216 on the
// main grid, core/oversampled_region.cpp:363-408 on a region grid.  Kahan sum
// over the point sources, added to the model.  Value I_tot * P(s (x - x0),
// s (y - y0)) (func_pointsource.cpp:220-229), rotated by PA for PointSourceRot
// (func_pointsource-rot.cpp:229-243); s = scales.s[c], the component's
// PointSource::oversamplingScale for this pass.
__global__ void __launch_bounds__(256) k_point_sources64(const CompF64 *__restrict__ comps, int nComp,
                                                         double *__restrict__ model, long pitch, Grid64 g,
                                                         PsfInterp<double> ip, PsScales scales) {
  __shared__ CompF64 sc[kMaxComponents];
  for (int i = threadIdx.x; i < nComp; i += blockDim.x) sc[i] = comps[i];
  __syncthreads();
  const long n = (long)g.nCols * g.nRows;
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long j = k % g.nCols, i = k / g.nCols;
  double x, y;
  if (!g.isRegion) {
    y = (double)(i - g.pr + 1);
    x = (double)(j - g.pc + 1);
  } else {
    y = g.y1 + g.off + (i - g.pr) * g.frac;
    x = g.x1 + g.off + (j - g.pc) * g.frac;
  }
  double s = 0.0, err = 0.0;
  for (int c = 0; c < nComp; c++) {
    const CompF64 &f = sc[c];
    if (!is_point_source(f.type)) continue;
    const double os = (double)scales.s[c];
    double xd = os * (x - f.x0), yd = os * (y - f.y0);
    if (f.type == F_POINTSOURCEROT) {
      const double xp = xd * f.cosPA + yd * f.sinPA;
      const double yp = -xd * f.sinPA + yd * f.cosPA;
      xd = xp;
      yd = yp;
    }
    const double v = f.a * psf_interp64(ip, xd, yd);
    const double adj = v - err;
    const double tmp = s + adj;
    err = (tmp - s) - adj;
    s = tmp;
  }
  model[i * pitch + j] += s;
}

cudaError_t launch_point_sources64(const CompF64 *comps, int nComp, double *model, long pitch, Grid64 g,
                                   PsfInterp<double> ip, const PsScales &scales, cudaStream_t st) {
  const long n = (long)g.nCols * g.nRows;
  if (n == 0) return cudaSuccess;
  k_point_sources64<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(comps, nComp, model, pitch, g, ip, scales);
  return cudaGetLastError();
}

// DownsampleAndReplace: core/downsample.cpp:54-109.  nRows_subregion uses the
// column count (core/downsample.cpp:79); the caller has checked the reads stay
// inside the region model.
__global__ void k_downsample64(const double *__restrict__ os, int nOC, int osPsfCols, int osPsfRows,
                               double *__restrict__ mainImg, int nMainCols, int i1, int j1, int nColsSub,
                               int nRowsSub, int scale) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nColsSub * nRowsSub) return;
  const int i_sub = t / nColsSub, j_sub = t % nColsSub;
  const int jj1 = j_sub * scale + osPsfCols;
  const int ii1 = i_sub * scale + osPsfRows;
  double b = 0.0;
  for (int ii = ii1; ii < ii1 + scale; ii++)
    for (int jj = jj1; jj < jj1 + scale; jj++) b += os[(long)ii * nOC + jj];
  const double area = scale * scale;
  mainImg[(long)(i1 + i_sub) * nMainCols + (j1 + j_sub)] = b / area;
}

cudaError_t launch_downsample64(const double *region, int nOC, int nOR, int osPsfCols, int osPsfRows,
                                double *mainImg, int nMainCols, int nMainRows, int mainPsfCols,
                                int mainPsfRows, int x1, int y1, int scale, cudaStream_t st) {
  (void)nOR;
  (void)nMainRows;
  const int j1 = x1 - 1 + mainPsfCols;
  const int i1 = y1 - 1 + mainPsfRows;
  const int nColsSub = (nOC - 2 * osPsfCols) / scale;
  const int nRowsSub = (nOC - 2 * osPsfRows) / scale;
  const int n = nColsSub * nRowsSub;
  if (n <= 0) return cudaSuccess;
  k_downsample64<<<(n + 127) / 128, 128, 0, st>>>(region, nOC, osPsfCols, osPsfRows, mainImg, nMainCols, i1, j1,
                                                  nColsSub, nRowsSub, scale);
  return cudaGetLastError();
}

// ------------------------------------------------------------- statistics
#define LOG_SMALL_VALUE 1.0e-25  // core/model_object.cpp:86

struct Term {
  double w, d, m, extra;
  long b;
};

__device__ __forceinline__ long model_index(const StatArgs64 &a, long b) {
  const long row = b / a.nDataCols;
  const long col = b - row * a.nDataCols;
  return (long)a.modelCols * (a.offR + row) + a.offC + col;
}

// weight for term b; UpdateWeightVector (core/model_object.cpp:1345-1381)
// when model-based errors are in use
__device__ __forceinline__ double term_weight(const StatArgs64 &a, long b, double m) {
  if (a.modelErrors && a.mask[b] > 0) {
    const double tf = m + a.sky;
    const double ns = tf / a.effGain + a.rnTerm;
    return 1.0 / sqrt(ns);
  }
  return a.weight[b];
}

// ComputeDeviates (core/model_object.cpp:1413-1496) and
// ComputePoissonMLRDeviate (core/model_object.cpp:1386-1401)
__global__ void k_deviates64(StatArgs64 a, double *__restrict__ dev, double *__restrict__ wOut) {
  const long z = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (z >= a.nz) return;
  const long b = a.boot ? a.boot[z] : z;
  const double m = a.model[model_index(a, b)];
  const double w = term_weight(a, b, m);
  if (wOut && a.modelErrors && !a.boot) wOut[b] = w;
  double r;
  if (a.kind == 2) {
    const double mv = a.effGain * (m + a.sky);
    const double dv = a.effGain * (a.data[b] + a.sky);
    const double lm = (mv <= 0) ? LOG_SMALL_VALUE : log(mv);
    r = sqrt(2.0 * w * fabs(mv - dv * lm + a.extra[b]));
  } else {
    r = w * (a.data[b] - m);
  }
  dev[z] = r;
}

cudaError_t launch_deviates64(const StatArgs64 &a, double *dev, double *wOut, cudaStream_t st) {
  if (a.nz <= 0) return cudaSuccess;
  k_deviates64<<<(unsigned)((a.nz + 255) / 256), 256, 0, st>>>(a, dev, wOut);
  return cudaGetLastError();
}

// ChiSquared (core/model_object.cpp:1633-1689) and CashStatistic (:1703-1775),
// first level: fixed grid, grid-stride terms, per-block partial state.
__global__ void __launch_bounds__(256) k_stat64_partial(StatArgs64 a, double *__restrict__ partials) {
  const long stride = (long)gridDim.x * blockDim.x;
  if (a.kind == 0) {
    Enorm e = {0, 0, 0, 0, 0};
    const double agiant = 1.304e19 / (double)(int)a.nz;
    for (long z = blockIdx.x * (long)blockDim.x + threadIdx.x; z < a.nz; z += stride) {
      const long b = a.boot ? a.boot[z] : z;
      const double m = a.model[model_index(a, b)];
      const double w = term_weight(a, b, m);
      enorm_add(e, w * (a.data[b] - m), agiant);
    }
    e = block_enorm(e);
    if (threadIdx.x == 0) {
      double *p = partials + blockIdx.x * 5;
      p[0] = e.s1; p[1] = e.x1; p[2] = e.s2; p[3] = e.s3; p[4] = e.x3;
    }
  } else {
    double s = 0.0;
    for (long z = blockIdx.x * (long)blockDim.x + threadIdx.x; z < a.nz; z += stride) {
      const long b = a.boot ? a.boot[z] : z;
      const double mv = a.effGain * (a.model[model_index(a, b)] + a.sky);
      const double dv = a.effGain * (a.data[b] + a.sky);
      const double lm = (mv <= 0) ? LOG_SMALL_VALUE : log(mv);
      s += a.weight[b] * (mv - dv * lm + a.extra[b]);
    }
    s = block_sum(s);
    if (threadIdx.x == 0) partials[blockIdx.x * 5] = s;
  }
}

__global__ void __launch_bounds__(256) k_stat64_final(const double *__restrict__ partials, int nPart, int kind,
                                                      double *__restrict__ result) {
  if (kind == 0) {
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
  } else {
    double s = 0.0;
    for (int i = threadIdx.x; i < nPart; i += blockDim.x) s += partials[i * 5];
    s = block_sum(s);
    if (threadIdx.x == 0) *result = 2.0 * s;
  }
}

cudaError_t launch_statistic64(const StatArgs64 &a, double *partials, double *result, cudaStream_t st) {
  k_stat64_partial<<<kStatBlocks, 256, 0, st>>>(a, partials);
  k_stat64_final<<<1, 256, 0, st>>>(partials, kStatBlocks, a.kind == 0 ? 0 : 1, result);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(256) k_fd_dot_partial(const double *__restrict__ d0,
                                                        const double *__restrict__ d1, long n, double invh,
                                                        double *__restrict__ partials) {
  const long stride = (long)gridDim.x * blockDim.x;
  double s = 0.0;
  for (long z = blockIdx.x * (long)blockDim.x + threadIdx.x; z < n; z += stride)
    s += d0[z] * ((d1[z] - d0[z]) * invh);
  s = block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x * 5] = s;
}

cudaError_t launch_fd_dot64(const double *dev0, const double *dev1, long n, double invh, double *partials,
                            double *result, cudaStream_t st) {
  k_fd_dot_partial<<<kStatBlocks, 256, 0, st>>>(dev0, dev1, n, invh, partials);
  k_stat64_final<<<1, 256, 0, st>>>(partials, kStatBlocks, 1, result);  // returns 2*sum
  return cudaGetLastError();
}

__global__ void k_crop64(const double *__restrict__ model, int modelCols, int offR, int offC, int nCols,
                         int nRows, double *__restrict__ out) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)nCols * nRows) return;
  const long r = t / nCols, c = t % nCols;
  out[t] = model[(long)modelCols * (offR + r) + offC + c];
}

cudaError_t launch_crop64(const double *model, int modelCols, int offR, int offC, int nCols, int nRows,
                          double *out, cudaStream_t st) {
  const long n = (long)nCols * nRows;
  if (n == 0) return cudaSuccess;
  k_crop64<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(model, modelCols, offR, offC, nCols, nRows, out);
  return cudaGetLastError();
}

// UpdateWeightVector (core/model_object.cpp:1345-1381): model-based weights
// for unmasked pixels, recomputed after every model image.
__global__ void k_update_weights64(const double *__restrict__ model, const double *__restrict__ mask,
                                   double *__restrict__ weight, long nData, int nDataCols, int modelCols,
                                   int offR, int offC, double effGain, double sky, double rnTerm) {
  const long z = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (z >= nData || !(mask[z] > 0)) return;
  const long row = z / nDataCols, col = z - row * nDataCols;
  const double tf = model[(long)modelCols * (offR + row) + offC + col] + sky;
  const double ns = tf / effGain + rnTerm;
  weight[z] = 1.0 / sqrt(ns);
}

cudaError_t launch_update_weights64(const double *model, const double *mask, double *weight, long nData,
                                    int nDataCols, int modelCols, int offR, int offC, double effGain, double sky,
                                    double rnTerm, cudaStream_t st) {
  if (nData <= 0) return cudaSuccess;
  k_update_weights64<<<(unsigned)((nData + 255) / 256), 256, 0, st>>>(model, mask, weight, nData, nDataCols,
                                                                        modelCols, offR, offC, effGain, sky, rnTerm);
  return cudaGetLastError();
}

__global__ void k_f64_to_f32(const double *__restrict__ in, float *__restrict__ out, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

cudaError_t launch_f64_to_f32(const double *in, float *out, long n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_f64_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

}  // namespace imfit
