// k_fast.cu -- batched FP32-evaluation / FP64-reduction path with the adjoint
// gradient.
//
// Per parameter vector b the statistic S(theta) and dS/dtheta are formed by
//   setup      FP64 per-component geometry and Sersic b_n      (FunctionObject::Setup)
//   eval_r2c   model window rows evaluated in FP32 (SFU lg2/ex2), subsampled
//              pixels summed warp-cooperatively, then the row FFT -- the model
//              image never goes to HBM                         (CreateModelImage pixel loop)
//   cols       column FFT x PSF spectrum x inverse column FFT  (Convolver::ConvolveImage)
//   region     oversampled region: same pipeline at k x resolution and a
//              fused block-average                             (OversampledRegion, DownsampleAndReplace)
//   stat_rows  inverse row FFT, statistic terms accumulated in FP64, the
//              adjoint seed g = dS/dM written and immediately row-FFT'd
//                                                              (ChiSquared / CashStatistic)
//   cols(conj) the adjoint: correlation of g with the PSF
//   grad_rows  inverse row FFT, then one pass over the window accumulating
//              r~ * dm/dtheta for every parameter (subsampled pixels again
//              warp-cooperative), FP64 per-block partials
//   reduce     deterministic final sums.
// The "valid" window W = N + P - 1 (rather than the reference's N + 2P model
// plus N + 3P - 1 padding) is exactly the set of model pixels the data
// crop depends on; constant backgrounds (FlatSky) are added after the
// convolution as I_sky * sum(PSF), which is what convolving a constant gives.
#include "kernels.h"
#include "fft.cuh"

namespace imfit {

struct WinDesc {
  int cols, rows;
  int isRegion;
  int xOrig, yOrig;  // main: IRAF x = col + xOrig, y = row + yOrig
  int x1, y1, offX, offY, scale;
  float startOff, frac;
  int specPitch;
  long specBatch;
  cplx<float> *spec;
};

__device__ __forceinline__ int floordiv(int a, int b) {
  int q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
  return q;
}

__device__ __forceinline__ void win_offsets(const WinDesc &w, const CompF32 &c, int row, int col, float &dx,
                                            float &dy) {
  int xi, yi;
  float xf = 0.f, yf = 0.f;
  if (!w.isRegion) {
    xi = col + w.xOrig;
    yi = row + w.yOrig;
  } else {
    const int tx = col + w.offX, ty = row + w.offY;
    const int qx = floordiv(tx, w.scale), qy = floordiv(ty, w.scale);
    xi = w.x1 + qx;
    yi = w.y1 + qy;
    xf = w.startOff + (float)(tx - qx * w.scale) * w.frac;
    yf = w.startOff + (float)(ty - qy * w.scale) * w.frac;
  }
  dx = (float)(xi - c.x0i) + (xf - c.x0r);
  dy = (float)(yi - c.y0i) + (yf - c.y0r);
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
__global__ void k_fast_setup(FastArgs a) {
  const int b = blockIdx.x;
  const double *p = a.params + (long)b * a.nParams;
  for (int c = threadIdx.x; c < a.nComp; c += blockDim.x) comp_setup32(a.comps[b * a.nComp + c], a.desc[c], p);
  if (threadIdx.x == 0) {
    double bg = 0.0;
    for (int c = 0; c < a.nComp; c++)
      if (a.desc[c].background) bg += p[a.desc[c].paramOffset];
    a.bgLevel[2 * b] = (float)(bg * a.psfSum);
    a.bgLevel[2 * b + 1] = (float)(bg * a.psfSumOs);
  }
}

cudaError_t fast_setup(const FastArgs &a, int nBatch, cudaStream_t st) {
  k_fast_setup<<<nBatch, 32, 0, st>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------ eval + row r2c
__global__ void __launch_bounds__(256) k_fast_eval_r2c(FastArgs a, WinDesc w, FFTPlan<float> plan,
                                                       const cplx<float> *__restrict__ twL, int rpb) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y;
  const int M = plan.n, ls = M + 1;
  CompF32 *sc = reinterpret_cast<CompF32 *>(smem);
  cplx<float> *bufA = reinterpret_cast<cplx<float> *>(sc + kMaxComponents);
  cplx<float> *bufB = bufA + rpb * ls;
  unsigned char *flags = reinterpret_cast<unsigned char *>(bufB + rpb * ls);
  const int nC = a.nComp;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) sc[i] = a.comps[b * nC + i];
  const int row0 = blockIdx.x * rpb;
  const int nl = min(rpb, w.rows - row0);
  __syncthreads();
  if (nl <= 0) return;
  const int twoM = 2 * M;
  // pass 1: one thread per complex point (two pixels)
  for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
    const int l = idx / M, k = idx - l * M;
    const int row = row0 + l;
    float v[2] = {0.f, 0.f};
    unsigned char f[2] = {0, 0};
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const int col = 2 * k + e;
      if (col < w.cols) {
        for (int c = 0; c < nC; c++) {
          const CompF32 &cc = sc[c];
          if (cc.type == F_FLATSKY) continue;
          float dx, dy;
          win_offsets(w, cc, row, col, dx, dy);
          const Geo g = geo32(cc, dx, dy);
          if (sub_count(cc, g) > 1) {
            f[e] = 1;
            continue;
          }
          v[e] += radial32(cc, g.r2);
        }
      }
    }
    bufA[l * ls + k] = {v[0], v[1]};
    flags[l * twoM + 2 * k] = f[0];
    flags[l * twoM + 2 * k + 1] = f[1];
  }
  __syncthreads();
  // pass 2: subsampled pixels, one warp per pixel
  {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int cpr = (twoM + 31) >> 5;
    for (int ch = wid; ch < nl * cpr; ch += nw) {
      const int l = ch / cpr, p0 = (ch - l * cpr) << 5;
      const int p = p0 + lane;
      unsigned mask = __ballot_sync(0xffffffffu, (p < twoM) && flags[l * twoM + p]);
      while (mask) {
        const int q = p0 + __ffs(mask) - 1;
        mask &= mask - 1;
        float tot = 0.f;
        for (int c = 0; c < nC; c++) {
          const CompF32 &cc = sc[c];
          if (cc.type == F_FLATSKY) continue;
          float dx, dy;
          win_offsets(w, cc, row0 + l, q, dx, dy);
          const Geo g = geo32(cc, dx, dy);
          const int ns = sub_count(cc, g);
          if (ns <= 1) continue;
          const float d = 1.f / ns;
          const float xs = dx - 0.5f + 0.5f * d, ys = dy - 0.5f + 0.5f * d;
          float s = 0.f;
          for (int t = lane; t < ns * ns; t += 32) {
            const int ii = t / ns, jj = t - ii * ns;
            const Geo gs = geo32(cc, xs + ii * d, ys + jj * d);
            s += radial32(cc, gs.r2);
          }
          tot += warp_sum(s) * (d * d);
        }
        if (lane == 0) {
          cplx<float> &z = bufA[l * ls + (q >> 1)];
          if (q & 1) z.y += tot; else z.x += tot;
        }
      }
    }
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, plan, nl, ls, 1, -1, false);
  cplx<float> *out = w.spec + (long)b * w.specBatch;
  for (int idx = threadIdx.x; idx < nl * (M + 1); idx += blockDim.x) {
    const int l = idx / (M + 1), k = idx - l * (M + 1);
    out[(long)(row0 + l) * w.specPitch + k] = r2c_post(Z + l * ls, k, M, twL);
  }
}

// ---------------------------------------- region: c2r + block average
__global__ void __launch_bounds__(256) k_fast_region_down(FastArgs a, FastGeom g, const cplx<float> *__restrict__ rspec,
                                                          FFTPlan<float> plan, const cplx<float> *__restrict__ twL) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y, s = blockIdx.x;  // replaced data row within the region
  const int k = g.rScale;
  const int M = plan.n, ls = M + 1;
  cplx<float> *bufX = reinterpret_cast<cplx<float> *>(smem);
  cplx<float> *bufA = bufX + k * ls;
  cplx<float> *bufB = bufA + k * ls;
  const cplx<float> *in = rspec + (long)b * g.rSpecBatch + (long)(s * k) * g.rSpecPitch;
  for (int idx = threadIdx.x; idx < k * (M + 1); idx += blockDim.x) {
    const int l = idx / (M + 1), kk = idx - l * (M + 1);
    bufX[l * ls + kk] = in[(long)l * g.rSpecPitch + kk];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < k * M; idx += blockDim.x) {
    const int l = idx / M, kk = idx - l * M;
    bufA[l * ls + kk] = c2r_pre(bufX + l * ls, kk, M, twL);
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, plan, k, ls, 1, +1, false);
  const float inv = 1.f / (float)(k * k);
  const float bg = a.bgLevel[2 * b + 1];
  for (int t = threadIdx.x; t < g.rCols; t += blockDim.x) {
    float acc = 0.f;
    for (int u = 0; u < k; u++)
      for (int v = 0; v < k; v++) {
        const int col = t * k + v;
        const cplx<float> z = Z[u * ls + (col >> 1)];
        acc += (col & 1) ? z.y : z.x;
      }
    a.regModel[((long)b * g.rRows + s) * g.rCols + t] = acc * inv + bg;
  }
}

// -------------------------- stat rows: c2r + statistic + g + g row r2c
__device__ __forceinline__ void stat_term(const FastArgs &a, long z, float m, double &S, float &gout) {
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
      S += (double)cnt * (double)r * (double)r / (double)V;
      gout = cnt * (-2.f * r / V - r * r / (V * V * a.effGain));
    } else {
      const float dev = w * (d - m);
      S += (double)cnt * (double)dev * (double)dev;
      gout = -2.f * cnt * w * dev;
    }
  } else {
    const float mv = a.effGain * (m + a.sky);
    const float dv = a.effGain * (d + a.sky);
    const float ex = a.extra ? a.extra[z] : 0.f;
    double term;
    float dterm;
    if (mv > 0.f) {
      if (ex != 0.f && dv > 0.f) {
        // (mv - dv ln mv) + (dv ln dv - dv) written without cancellation
        const float del = (mv - dv) / dv;
        term = (double)(mv - dv) - (double)dv * (double)log1pf(del);
      } else {
        term = (double)mv - (double)dv * (double)logf(mv) + (double)ex;
      }
      dterm = a.effGain * (1.f - dv / mv);
    } else {
      term = (double)mv - (double)dv * 1.0e-25 + (double)ex;
      dterm = a.effGain;
    }
    S += 2.0 * (double)cnt * (double)w * term;
    gout = 2.f * cnt * w * dterm;
  }
}

__global__ void __launch_bounds__(256) k_fast_stat_rows(FastArgs a, FastGeom g, FFTPlan<float> plan,
                                                        const cplx<float> *__restrict__ twL, int rpb, int wantGrad) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y;
  const int M = plan.n, ls = M + 1;
  cplx<float> *bufX = reinterpret_cast<cplx<float> *>(smem);
  cplx<float> *bufA = bufX + rpb * ls;
  cplx<float> *bufB = bufA + rpb * ls;
  __shared__ double red[2][32];
  const int row0 = blockIdx.x * rpb;
  const int nl = min(rpb, g.nDataRows - row0);
  cplx<float> *spec = reinterpret_cast<cplx<float> *>(a.spec) + (long)b * g.specBatch;
  double S = 0.0, SG = 0.0;
  if (nl > 0) {
    for (int idx = threadIdx.x; idx < nl * (M + 1); idx += blockDim.x) {
      const int l = idx / (M + 1), k = idx - l * (M + 1);
      bufX[l * ls + k] = spec[(long)(row0 + l) * g.specPitch + k];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
      const int l = idx / M, k = idx - l * M;
      bufA[l * ls + k] = c2r_pre(bufX + l * ls, k, M, twL);
    }
    __syncthreads();
    cplx<float> *Z = block_fft(bufA, bufB, plan, nl, ls, 1, +1, false);
    cplx<float> *G = (Z == bufA) ? bufB : bufA;
    const float bg = a.bgLevel[2 * b];
    // one thread per complex point = two data columns
    for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
      const int l = idx / M, k = idx - l * M;
      const int row = row0 + l;
      const cplx<float> zz = Z[l * ls + k];
      float gv[2] = {0.f, 0.f};
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const int col = 2 * k + e;
        if (col >= g.nDataCols) continue;
        const long zi = (long)row * g.nDataCols + col;
        float m = (e ? zz.y : zz.x) + bg;
        bool inReg = false;
        long ri = 0;
        if (g.hasRegion) {
          const int rr = row - g.ry0, rc = col - g.rx0;
          if (rr >= 0 && rr < g.rRows && rc >= 0 && rc < g.rCols) {
            inReg = true;
            ri = ((long)b * g.rRows + rr) * g.rCols + rc;
            m = a.regModel[ri];
          }
        }
        if (a.modelOut) a.modelOut[(long)b * g.nDataRows * g.nDataCols + zi] = m;
        float gz;
        stat_term(a, zi, m, S, gz);
        SG += (double)gz * (double)(inReg ? a.psfSumOs : a.psfSum);
        if (inReg) {
          if (wantGrad) a.regG[ri] = gz;
          gz = 0.f;
        }
        gv[e] = gz;
      }
      G[l * ls + k] = {gv[0], gv[1]};
    }
    __syncthreads();
    if (wantGrad) {
      cplx<float> *other = (G == bufA) ? bufB : bufA;
      cplx<float> *R = block_fft(G, other, plan, nl, ls, 1, -1, false);
      for (int idx = threadIdx.x; idx < nl * (M + 1); idx += blockDim.x) {
        const int l = idx / (M + 1), k = idx - l * (M + 1);
        spec[(long)(row0 + l) * g.specPitch + k] = r2c_post(R + l * ls, k, M, twL);
      }
    }
  }
  // block reduction of (S, SG)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  S = warp_sum_d(S);
  SG = warp_sum_d(SG);
  if (lane == 0) {
    red[0][wid] = S;
    red[1][wid] = SG;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
      s0 += red[0][i];
      s1 += red[1][i];
    }
    double *p = a.statPart + ((long)b * a.nStatBlocks + blockIdx.x) * 2;
    p[0] = s0;
    p[1] = s1;
  }
}

// --------------------------- region adjoint seed: g/k^2 on subpixels, r2c
__global__ void __launch_bounds__(256) k_fast_region_g_r2c(FastArgs a, FastGeom g, cplx<float> *__restrict__ rspec,
                                                           FFTPlan<float> plan, const cplx<float> *__restrict__ twL) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y, u = blockIdx.x;  // subpixel row
  const int M = plan.n, ls = M + 1;
  cplx<float> *bufA = reinterpret_cast<cplx<float> *>(smem);
  cplx<float> *bufB = bufA + ls;
  const int k = g.rScale;
  const float inv = 1.f / (float)(k * k);
  const float *gr = a.regG + ((long)b * g.rRows + u / k) * g.rCols;
  for (int kk = threadIdx.x; kk < M; kk += blockDim.x) {
    const int c0 = 2 * kk, c1 = 2 * kk + 1;
    cplx<float> z;
    z.x = (c0 < g.rSubCols) ? gr[c0 / k] * inv : 0.f;
    z.y = (c1 < g.rSubCols) ? gr[c1 / k] * inv : 0.f;
    bufA[kk] = z;
  }
  __syncthreads();
  cplx<float> *Z = block_fft(bufA, bufB, plan, 1, ls, 1, -1, false);
  cplx<float> *out = rspec + (long)b * g.rSpecBatch + (long)u * g.rSpecPitch;
  for (int kk = threadIdx.x; kk <= M; kk += blockDim.x) out[kk] = r2c_post(Z, kk, M, twL);
}

// ---------------------------------------- gradient pass over the window
__global__ void __launch_bounds__(256) k_fast_grad_rows(FastArgs a, WinDesc w, FFTPlan<float> plan,
                                                        const cplx<float> *__restrict__ twL, int rpb,
                                                        double *__restrict__ gradPart, int nBlocksTotal,
                                                        int blockBase) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.y;
  const int M = plan.n, ls = M + 1;
  CompF32 *sc = reinterpret_cast<CompF32 *>(smem);
  double *gsm = reinterpret_cast<double *>(sc + kMaxComponents);
  cplx<float> *bufX = reinterpret_cast<cplx<float> *>(gsm + kMaxParams);
  cplx<float> *bufA = bufX + rpb * ls;
  cplx<float> *bufB = bufA + rpb * ls;
  unsigned char *flags = reinterpret_cast<unsigned char *>(bufB + rpb * ls);
  __shared__ float red[8][8];
  const int nC = a.nComp, nP = a.nParams;
  for (int i = threadIdx.x; i < nC; i += blockDim.x) sc[i] = a.comps[b * nC + i];
  for (int i = threadIdx.x; i < nP; i += blockDim.x) gsm[i] = 0.0;
  const int row0 = blockIdx.x * rpb;
  const int nl = min(rpb, w.rows - row0);
  const cplx<float> *spec = w.spec + (long)b * w.specBatch;
  for (int idx = threadIdx.x; idx < max(nl, 0) * (M + 1); idx += blockDim.x) {
    const int l = idx / (M + 1), k = idx - l * (M + 1);
    bufX[l * ls + k] = spec[(long)(row0 + l) * w.specPitch + k];
  }
  __syncthreads();
  if (nl > 0) {
    for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
      const int l = idx / M, k = idx - l * M;
      bufA[l * ls + k] = c2r_pre(bufX + l * ls, k, M, twL);
    }
    __syncthreads();
    cplx<float> *Z = block_fft(bufA, bufB, plan, nl, ls, 1, +1, false);
    const float *rt = reinterpret_cast<const float *>(Z);  // r~ of (l, col) at rt[2*(l*ls) + col]
    const int twoM = 2 * M;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c = 0; c < nC; c++) {
      const CompF32 &cc = sc[c];
      if (cc.type == F_FLATSKY) continue;
      float acc[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      float o[7];
      for (int idx = threadIdx.x; idx < nl * twoM; idx += blockDim.x) {
        const int l = idx / twoM, col = idx - l * twoM;
        unsigned char f = 0;
        if (col < w.cols) {
          const float r = rt[2 * l * ls + col];
          float dx, dy;
          win_offsets(w, cc, row0 + l, col, dx, dy);
          const Geo g = geo32(cc, dx, dy);
          if (sub_count(cc, g) > 1) {
            f = 1;
          } else if (r != 0.f) {
            const int np = radial_grad32(cc, g, r, o);
#pragma unroll
            for (int q = 0; q < 7; q++)
              if (q < 2 + np) acc[q] += o[q];
          }
        }
        flags[l * twoM + col] = f;
      }
      __syncthreads();
      const int cprr = (twoM + 31) >> 5;
      for (int ch = wid; ch < nl * cprr; ch += nw) {
        const int l = ch / cprr, p0 = (ch - l * cprr) << 5;
        const int p = p0 + lane;
        unsigned mask = __ballot_sync(0xffffffffu, (p < twoM) && flags[l * twoM + p]);
        while (mask) {
          const int q = p0 + __ffs(mask) - 1;
          mask &= mask - 1;
          const float r = rt[2 * l * ls + q];
          float dx, dy;
          win_offsets(w, cc, row0 + l, q, dx, dy);
          const Geo g = geo32(cc, dx, dy);
          const int ns = sub_count(cc, g);
          const float d = 1.f / ns;
          const float scale = r * d * d;
          const float xs = dx - 0.5f + 0.5f * d, ys = dy - 0.5f + 0.5f * d;
          for (int t = lane; t < ns * ns; t += 32) {
            const int ii = t / ns, jj = t - ii * ns;
            const Geo gs = geo32(cc, xs + ii * d, ys + jj * d);
            const int np = radial_grad32(cc, gs, scale, o);
#pragma unroll
            for (int qq = 0; qq < 7; qq++)
              if (qq < 2 + np) acc[qq] += o[qq];
          }
        }
      }
      // block reduction of acc[0..6]
#pragma unroll
      for (int q = 0; q < 7; q++) acc[q] = warp_sum(acc[q]);
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < 7; q++) red[wid][q] = acc[q];
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double t[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int i = 0; i < nw; i++)
          for (int q = 0; q < 7; q++) t[q] += (double)red[i][q];
        gsm[cc.x0Index] += t[0];
        gsm[cc.x0Index + 1] += t[1];
        const int npf = a.desc[c].nParams;
        for (int q = 0; q < npf && q < 5; q++) gsm[cc.paramOffset + q] += t[2 + q];
      }
      __syncthreads();
    }
  }
  __syncthreads();
  double *out = gradPart + ((long)b * nBlocksTotal + blockBase + blockIdx.x) * nP;
  for (int i = threadIdx.x; i < nP; i += blockDim.x) out[i] = gsm[i];
}

// ------------------------------------------------------------- reduce
__global__ void __launch_bounds__(256) k_fast_reduce(FastArgs a, int nGradBlocks, int wantGrad) {
  const int b = blockIdx.x;
  __shared__ double sh[32];
  // statistic
  double s = 0.0, sg = 0.0;
  for (int i = threadIdx.x; i < a.nStatBlocks; i += blockDim.x) {
    const double *p = a.statPart + ((long)b * a.nStatBlocks + i) * 2;
    s += p[0];
    sg += p[1];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  s = warp_sum_d(s);
  sg = warp_sum_d(sg);
  if (lane == 0) sh[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < nw; i++) t += sh[i];
    a.stat[b] = t;
  }
  __syncthreads();
  if (lane == 0) sh[wid] = sg;
  __syncthreads();
  double sgt = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < nw; i++) sgt += sh[i];
  __syncthreads();
  if (threadIdx.x == 0) sh[0] = sgt;
  __syncthreads();
  sgt = sh[0];
  if (!wantGrad) return;
  for (int j = threadIdx.x; j < a.nParams; j += blockDim.x) {
    double t = 0.0;
    for (int i = 0; i < nGradBlocks; i++) t += a.gradPart[((long)b * nGradBlocks + i) * a.nParams + j];
    a.grad[(long)b * a.nParams + j] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int c = 0; c < a.nComp; c++)
      if (a.desc[c].background) a.grad[(long)b * a.nParams + a.desc[c].paramOffset] = sgt;
  }
}

// ------------------------------------------------------------ launchers
static FFTPlan<float> plan32(const FFTLen &L, bool half) {
  FFTPlan<float> p;
  const FFTTable &t = half ? L.half : L.full;
  p.n = t.n;
  p.npass = t.npass;
  for (int i = 0; i < kMaxRadixPasses; i++) p.radix[i] = t.radix[i];
  p.tw = reinterpret_cast<const cplx<float> *>(t.tw32);
  return p;
}

static int fast_rpb(int M) {
  // ~40 KB of complex line buffers per CTA
  int r = (40 * 1024) / (3 * (M + 1) * 8);
  if (r < 1) r = 1;
  if (r > 4) r = 4;
  return r;
}

int fast_stat_blocks(const FastGeom &g) {
  const int M = (g.specPitch - 1);
  const int rpb = fast_rpb(M);
  return (g.nDataRows + rpb - 1) / rpb;
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
  w.startOff = g.rStartOff;
  w.frac = g.rFrac;
  w.specPitch = g.rSpecPitch;
  w.specBatch = g.rSpecBatch;
  w.spec = reinterpret_cast<cplx<float> *>(rspec);
  return w;
}

int fast_grad_blocks(const FastGeom &g) {
  const int rpb = fast_rpb(g.specPitch - 1);
  return (g.winRows + rpb - 1) / rpb;
}

int fast_reg_grad_blocks(const FastGeom &g) {
  if (!g.hasRegion) return 0;
  const int rpb = fast_rpb(g.rSpecPitch - 1);
  return (g.rWinRows + rpb - 1) / rpb;
}

template <typename K>
static void ensure_smem(K kern, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

static cudaError_t launch_eval(const FastArgs &a, const WinDesc &w, const FFTLen &L, int nBatch, cudaStream_t st) {
  const int M = L.half.n;
  const int rpb = fast_rpb(M);
  const size_t sm = sizeof(CompF32) * kMaxComponents + sizeof(cplx<float>) * 2 * rpb * (M + 1) + (size_t)rpb * 2 * M + 16;
  ensure_smem(k_fast_eval_r2c, sm);
  dim3 grid((w.rows + rpb - 1) / rpb, nBatch);
  k_fast_eval_r2c<<<grid, 256, sm, st>>>(a, w, plan32(L, true), reinterpret_cast<const cplx<float> *>(L.twL32), rpb);
  return cudaGetLastError();
}

static cudaError_t launch_grad(const FastArgs &a, const WinDesc &w, const FFTLen &L, int nBatch, int nBlocksTotal,
                               int blockBase, cudaStream_t st) {
  const int M = L.half.n;
  const int rpb = fast_rpb(M);
  const size_t sm = sizeof(CompF32) * kMaxComponents + sizeof(double) * kMaxParams +
                    sizeof(cplx<float>) * 3 * rpb * (M + 1) + (size_t)rpb * 2 * M + 16;
  ensure_smem(k_fast_grad_rows, sm);
  dim3 grid((w.rows + rpb - 1) / rpb, nBatch);
  k_fast_grad_rows<<<grid, 256, sm, st>>>(a, w, plan32(L, true), reinterpret_cast<const cplx<float> *>(L.twL32), rpb,
                                          a.gradPart, nBlocksTotal, blockBase);
  return cudaGetLastError();
}

static void mark(const FastPlan &p, const char *name, cudaStream_t st) {
  StageTimer *t = p.timer;
  if (!t || t->n >= StageTimer::kMax) return;
  // while the stream is being captured the record must be External to become an
  // event-record node of the graph; outside capture that flag is not allowed
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cs);
  if (cs == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(t->ev[t->n], st, cudaEventRecordExternal);
  else
    cudaEventRecord(t->ev[t->n], st);
  t->names[t->n] = name;
  t->n++;
}

cudaError_t fast_forward(const FastPlan &p, const FastArgs &a, int nBatch, bool wantGrad, cudaStream_t st) {
  const FastGeom &g = p.g;
  if (p.timer) p.timer->n = 0;
  mark(p, "start", st);
  cudaError_t e = fast_setup(a, nBatch, st);
  if (e) return e;
  mark(p, "setup", st);
  // main window -> spectrum
  e = launch_eval(a, main_win(g, a.spec), *p.Lx, nBatch, st);
  if (e) return e;
  mark(p, "eval_r2c", st);
  const float scale = 1.f / ((float)p.Lx->L * (float)p.Ly->L);
  e = launch_cols<float>(a.spec, g.specPitch, g.specBatch, p.Lx->L / 2 + 1, g.winRows, g.nDataRows, p.H, p.hPitch,
                         *p.Ly, scale, 1, nBatch, st);
  if (e) return e;
  mark(p, "cols_conv", st);
  if (g.hasRegion) {
    e = launch_eval(a, region_win(g, a.rspec), *p.Rx, nBatch, st);
    if (e) return e;
    mark(p, "region_eval_r2c", st);
    const float rscale = 1.f / ((float)p.Rx->L * (float)p.Ry->L);
    e = launch_cols<float>(a.rspec, g.rSpecPitch, g.rSpecBatch, p.Rx->L / 2 + 1, g.rWinRows, g.rSubRows, p.Hr,
                           p.hrPitch, *p.Ry, rscale, 1, nBatch, st);
    if (e) return e;
    mark(p, "region_cols_conv", st);
    const int M = p.Rx->half.n;
    const size_t sm = sizeof(cplx<float>) * 3 * g.rScale * (M + 1);
    ensure_smem(k_fast_region_down, sm);
    k_fast_region_down<<<dim3(g.rRows, nBatch), 256, sm, st>>>(a, g, reinterpret_cast<const cplx<float> *>(a.rspec),
                                                               plan32(*p.Rx, true),
                                                               reinterpret_cast<const cplx<float> *>(p.Rx->twL32));
    e = cudaGetLastError();
    if (e) return e;
    mark(p, "region_down", st);
  }
  {
    const int M = p.Lx->half.n;
    const int rpb = fast_rpb(M);
    const size_t sm = sizeof(cplx<float>) * 3 * rpb * (M + 1);
    ensure_smem(k_fast_stat_rows, sm);
    dim3 grid((g.nDataRows + rpb - 1) / rpb, nBatch);
    k_fast_stat_rows<<<grid, 256, sm, st>>>(a, g, plan32(*p.Lx, true),
                                            reinterpret_cast<const cplx<float> *>(p.Lx->twL32), rpb, wantGrad ? 1 : 0);
    e = cudaGetLastError();
    if (e) return e;
    mark(p, "stat_rows", st);
  }
  if (!wantGrad) {
    k_fast_reduce<<<nBatch, 256, 0, st>>>(a, 0, 0);
    e = cudaGetLastError();
    mark(p, "reduce", st);
    return e;
  }
  return fast_adjoint(p, a, nBatch, st);
}

cudaError_t fast_adjoint(const FastPlan &p, const FastArgs &a, int nBatch, cudaStream_t st) {
  const FastGeom &g = p.g;
  cudaError_t e;
  const float scale = 1.f / ((float)p.Lx->L * (float)p.Ly->L);
  e = launch_cols<float>(a.spec, g.specPitch, g.specBatch, p.Lx->L / 2 + 1, g.nDataRows, g.winRows, p.H, p.hPitch,
                         *p.Ly, scale, 2, nBatch, st);
  if (e) return e;
  mark(p, "cols_adjoint", st);
  const int nMain = fast_grad_blocks(g), nReg = fast_reg_grad_blocks(g);
  const int nTot = nMain + nReg;
  e = launch_grad(a, main_win(g, a.spec), *p.Lx, nBatch, nTot, 0, st);
  if (e) return e;
  mark(p, "grad_rows", st);
  if (g.hasRegion) {
    const int M = p.Rx->half.n;
    const size_t sm = sizeof(cplx<float>) * 2 * (M + 1);
    k_fast_region_g_r2c<<<dim3(g.rSubRows, nBatch), 256, sm, st>>>(
        a, g, reinterpret_cast<cplx<float> *>(a.rspec), plan32(*p.Rx, true),
        reinterpret_cast<const cplx<float> *>(p.Rx->twL32));
    e = cudaGetLastError();
    if (e) return e;
    mark(p, "region_g_r2c", st);
    const float rscale = 1.f / ((float)p.Rx->L * (float)p.Ry->L);
    e = launch_cols<float>(a.rspec, g.rSpecPitch, g.rSpecBatch, p.Rx->L / 2 + 1, g.rSubRows, g.rWinRows, p.Hr,
                           p.hrPitch, *p.Ry, rscale, 2, nBatch, st);
    if (e) return e;
    mark(p, "region_cols_adjoint", st);
    e = launch_grad(a, region_win(g, a.rspec), *p.Rx, nBatch, nTot, nMain, st);
    if (e) return e;
    mark(p, "region_grad_rows", st);
  }
  k_fast_reduce<<<nBatch, 256, 0, st>>>(a, nTot, 1);
  e = cudaGetLastError();
  mark(p, "reduce", st);
  return e;
}

}  // namespace imfit
