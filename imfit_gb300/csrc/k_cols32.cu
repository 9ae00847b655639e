// k_cols32.cu -- column pass of the FP32 convolution (fast path).
//
// The middle step of Convolver::ConvolveImage (core/convolver.cpp:365-411):
// for each group of CPB adjacent half-spectrum columns, the column FFT, the
// multiplication by the cached PSF spectrum (or its conjugate: the adjoint
// correlation) with the 1/(Lx Ly) rescale, and the inverse column FFT, with
// one read and one write of the spectrum.
//
// Memory side (what the per-kernel profile showed to be the limit: long
// scoreboard stalls on one dependent 8-byte load per thread per element and
// a second round of PSF-spectrum loads after the forward FFT):
//   * every global read of the CTA -- the column group, the PSF spectrum's
//     matching columns and the twiddle table -- is issued at once as
//     cp.async copies into shared memory, so their latencies overlap each
//     other and the PSF spectrum arrives while the forward FFT runs;
//   * rows are moved in 16-byte pieces (two complex values; the spectrum
//     and PSF-spectrum pitches are even, so every piece is 16-byte aligned),
//     and written back with 16-byte vector stores;
//   * the FFT passes read their twiddles from the shared-memory copy.
// Rows at or beyond nRowsIn are the implicit zero padding and are never read.
#include "kernels.h"
#include "fft.cuh"

namespace imfit {

namespace {

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Copy the first `pairs` 16-byte pieces (complex pairs) of CPB columns of
// one row, zero the rest of the group; CPB == 1 moves one 8-byte value.
template <int CPB>
__device__ __forceinline__ void load_row(cplx<float> *dst, const cplx<float> *src, int pairs) {
  if constexpr (CPB == 1) {
    cp_async8(dst, src);
  } else {
#pragma unroll
    for (int q = 0; q < CPB / 2; q++) {
      if (q < pairs)
        cp_async16(dst + 2 * q, src + 2 * q);
      else
        *reinterpret_cast<float4 *>(dst + 2 * q) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

template <int CPB>
__device__ __forceinline__ void zero_row(cplx<float> *dst) {
  if constexpr (CPB == 1) {
    *dst = cplx<float>{0.f, 0.f};
  } else {
#pragma unroll
    for (int q = 0; q < CPB / 2; q++) *reinterpret_cast<float4 *>(dst + 2 * q) = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

template <int CPB>
__device__ __forceinline__ void store_row(cplx<float> *dst, const cplx<float> *src, int pairs) {
  if constexpr (CPB == 1) {
    *dst = *src;
  } else {
#pragma unroll
    for (int q = 0; q < CPB / 2; q++)
      if (q < pairs) *reinterpret_cast<float4 *>(dst + 2 * q) = *reinterpret_cast<const float4 *>(src + 2 * q);
  }
}

}  // namespace

// Column group body, shared with the ragged cutout kernels: the CPB columns
// starting at c0 of the spectrum `spec` (pitch, Ly = plan.n rows, nColsC
// columns), H (hPitch) the PSF spectrum of the same geometry, in the dynamic
// shared memory smem_raw (cols32_smem bytes: twiddles, two FFT buffers of
// padded_len(Ly * CPB) elements, the PSF columns).
// MODE 1: multiply by H (convolution); MODE 2: by conj(H) (adjoint correlation).
template <int MODE, int CPB>
__device__ __forceinline__ void cols_group(unsigned char *smem_raw, cplx<float> *spec, long pitch, int nColsC,
                                           int nRowsIn, int nRowsOut, const cplx<float> *H, long hPitch,
                                           const FFTPlan<float> &plan, float scale, int c0) {
  const int Ly = plan.n;
  const int bufLen = padded_len(Ly * CPB, 2);
  cplx<float> *tw = reinterpret_cast<cplx<float> *>(smem_raw);
  cplx<float> *bufA = tw + Ly;
  cplx<float> *bufB = bufA + bufLen;
  cplx<float> *bufH = bufB + bufLen;
  const int nl = min(CPB, nColsC - c0);
  if (nl <= 0) return;
  const int pairs = (nl + 1) >> 1;
  const bool padFirst = plan.padFirst != 0;
  spec += c0;
  H += c0;
  // all global reads of the CTA in flight at once
  for (int t = threadIdx.x; t < Ly; t += blockDim.x) {
    if (t < nRowsIn)
      load_row<CPB>(bufA + (long)t * CPB, spec + (long)t * pitch, pairs);
    else
      zero_row<CPB>(bufA + (long)t * CPB);
    load_row<CPB>(bufH + (long)t * CPB, H + (long)t * hPitch, pairs);
  }
  for (int i = threadIdx.x; 2 * i < Ly; i += blockDim.x) cp_async16(tw + 2 * i, plan.tw + 2 * i);
  cp_async_wait_all();
  __syncthreads();
  cplx<float> *X = padFirst ? block_fft<float, true>(bufA, bufB, plan, CPB, 1, CPB, -1, true, tw)
                            : block_fft<float, false>(bufA, bufB, plan, CPB, 1, CPB, -1, true, tw);
  for (int idx = threadIdx.x; idx < Ly * CPB; idx += blockDim.x) {
    cplx<float> h = bufH[idx];
    if (MODE == 2) h.y = -h.y;
    cplx<float> v = cmul(X[idx], h);
    X[idx] = {v.x * scale, v.y * scale};
  }
  __syncthreads();
  cplx<float> *other = (X == bufA) ? bufB : bufA;
  cplx<float> *Y = padFirst ? block_fft<float, true>(X, other, plan, CPB, 1, CPB, +1, true, tw)
                            : block_fft<float, false>(X, other, plan, CPB, 1, CPB, +1, true, tw);
  pdl_trigger();
  for (int t = threadIdx.x; t < nRowsOut; t += blockDim.x)
    store_row<CPB>(spec + (long)t * pitch, Y + (long)t * CPB, pairs);
}

namespace {

__device__ __forceinline__ int pad_rt(int i, int pad) { return i + pad * (i >> 4); }

template <int R>
__device__ __forceinline__ void dft_r(cplx<float> *v, int s) {
  if (R == 2) dft2(v);
  if (R == 3) dft3(v, s);
  if (R == 4) dft4(v, s);
  if (R == 5) dft5(v, s);
  if (R == 7) dft7(v, s);
  if (R == 8) dft8(v, s);
  if (R == 9) dft9(v, s);
}

// The forward transform's last pass (radix R, span n / R), the product with
// the PSF spectrum and the inverse transform's first pass (same radix: the
// inverse runs the radices in reverse order, span 1, no twiddles), in
// registers: thread (j, l) holds exactly the R values the inverse's first
// butterfly needs, so the spectrum between the two transforms never goes
// to shared memory.  pin / pout: padding of the source / destination layout.
template <int MODE, int CPB, int R>
__device__ void fused_mid(const cplx<float> *X, cplx<float> *Y, const cplx<float> *__restrict__ H, long hPitch,
                          int nl, int n, int pin, int pout, const cplx<float> *tw, float scale) {
  const int m = n / R;
  for (int idx = threadIdx.x; idx < m * CPB; idx += blockDim.x) {
    const int j = idx / CPB, l = idx - j * CPB;
    // the PSF spectrum's values for this thread, read from global memory (it
    // is shared by every vector of the batch and stays in L2) while the
    // butterfly runs
    cplx<float> hv[R];
#pragma unroll
    for (int t = 0; t < R; t++) hv[t] = (l < nl) ? H[(long)(j + t * m) * hPitch + l] : cplx<float>{0.f, 0.f};
    cplx<float> v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = X[pad_rt((j + r * m) * CPB + l, pin)];
    if (j != 0) {
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], twiddle(tw, (r - 1) * m + j, -1));
    }
    dft_r<R>(v, -1);
#pragma unroll
    for (int t = 0; t < R; t++) {
      cplx<float> h = hv[t];
      if (MODE == 2) h.y = -h.y;
      const cplx<float> z = cmul(v[t], h);
      v[t] = {z.x * scale, z.y * scale};
    }
    dft_r<R>(v, +1);
#pragma unroll
    for (int t = 0; t < R; t++) Y[pad_rt((j * R + t) * CPB + l, pout)] = v[t];
  }
}

// The inverse transform's last pass (radix R, span n / R), written straight
// to the spectrum rows j + t n / R below nRowsOut (columns below nl).
template <int CPB, int R>
__device__ void last_to_global(const cplx<float> *X, cplx<float> *spec, long pitch, int n, int pin,
                               const cplx<float> *tw, int nRowsOut, int nl) {
  const int m = n / R;
  for (int idx = threadIdx.x; idx < m * CPB; idx += blockDim.x) {
    const int j = idx / CPB, l = idx - j * CPB;
    cplx<float> v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = X[pad_rt((j + r * m) * CPB + l, pin)];
    if (j != 0) {
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], twiddle(tw, (r - 1) * m + j, +1));
    }
    dft_r<R>(v, +1);
    if (l < nl) {
#pragma unroll
      for (int t = 0; t < R; t++)
        if (j + t * m < nRowsOut) spec[(long)(j + t * m) * pitch + l] = v[t];
    }
  }
}

template <int MODE, int CPB>
__device__ void fused_mid_r(int R, const cplx<float> *X, cplx<float> *Y, const cplx<float> *H, long hPitch, int nl,
                            int n, int pin, int pout, const cplx<float> *tw, float scale) {
  switch (R) {
    case 2: fused_mid<MODE, CPB, 2>(X, Y, H, hPitch, nl, n, pin, pout, tw, scale); break;
    case 3: fused_mid<MODE, CPB, 3>(X, Y, H, hPitch, nl, n, pin, pout, tw, scale); break;
    case 4: fused_mid<MODE, CPB, 4>(X, Y, H, hPitch, nl, n, pin, pout, tw, scale); break;
    case 5: fused_mid<MODE, CPB, 5>(X, Y, H, hPitch, nl, n, pin, pout, tw, scale); break;
    case 7: fused_mid<MODE, CPB, 7>(X, Y, H, hPitch, nl, n, pin, pout, tw, scale); break;
    case 9: fused_mid<MODE, CPB, 9>(X, Y, H, hPitch, nl, n, pin, pout, tw, scale); break;
    default: fused_mid<MODE, CPB, 8>(X, Y, H, hPitch, nl, n, pin, pout, tw, scale); break;
  }
}

template <int CPB>
__device__ void last_to_global_r(int R, const cplx<float> *X, cplx<float> *spec, long pitch, int n, int pin,
                                 const cplx<float> *tw, int nRowsOut, int nl) {
  switch (R) {
    case 2: last_to_global<CPB, 2>(X, spec, pitch, n, pin, tw, nRowsOut, nl); break;
    case 3: last_to_global<CPB, 3>(X, spec, pitch, n, pin, tw, nRowsOut, nl); break;
    case 4: last_to_global<CPB, 4>(X, spec, pitch, n, pin, tw, nRowsOut, nl); break;
    case 5: last_to_global<CPB, 5>(X, spec, pitch, n, pin, tw, nRowsOut, nl); break;
    case 7: last_to_global<CPB, 7>(X, spec, pitch, n, pin, tw, nRowsOut, nl); break;
    case 9: last_to_global<CPB, 9>(X, spec, pitch, n, pin, tw, nRowsOut, nl); break;
    default: last_to_global<CPB, 8>(X, spec, pitch, n, pin, tw, nRowsOut, nl); break;
  }
}

// One Stockham pass over the CPB interleaved columns (element t of column l at
// t * CPB + l), CPB known at compile time so the line index is a shift and
// the strided addresses are running sums; pin / pout: padding (0 or 2) of
// the source / destination layout.
template <int CPB, int R>
__device__ __forceinline__ void col_pass(const cplx<float> *__restrict__ src, cplx<float> *__restrict__ dst, int n,
                                         int Ns, int pin, int pout, const cplx<float> *__restrict__ tw, int s) {
  const int m = n / R;
  const FastDiv byNs(Ns);
  for (int idx = threadIdx.x; idx < m * CPB; idx += blockDim.x) {
    const int j = idx / CPB, l = idx - j * CPB;
    const int k = j - byNs.div(j) * Ns;
    cplx<float> v[R];
    if (pin) {
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = src[pad_rt(idx + r * m * CPB, pin)];
    } else {
      const cplx<float> *in = src + idx;
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = in[r * m * CPB];
    }
    if (k != 0) {
      const cplx<float> *tk = tw + k;
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], twiddle(tk, (r - 1) * Ns, s));
    }
    dft_r<R>(v, s);
    const int o = ((j - k) * R + k) * CPB + l;
    if (pout) {
#pragma unroll
      for (int t = 0; t < R; t++) dst[pad_rt(o + t * Ns * CPB, pout)] = v[t];
    } else {
      cplx<float> *out = dst + o;
#pragma unroll
      for (int t = 0; t < R; t++) out[t * Ns * CPB] = v[t];
    }
  }
}

template <int CPB>
__device__ __forceinline__ void mid_pass(int R, const cplx<float> *src, cplx<float> *dst, int n, int Ns, int pin,
                                         int pout, const cplx<float> *tw, int s) {
  switch (R) {
    case 2: col_pass<CPB, 2>(src, dst, n, Ns, pin, pout, tw, s); break;
    case 3: col_pass<CPB, 3>(src, dst, n, Ns, pin, pout, tw, s); break;
    case 4: col_pass<CPB, 4>(src, dst, n, Ns, pin, pout, tw, s); break;
    case 5: col_pass<CPB, 5>(src, dst, n, Ns, pin, pout, tw, s); break;
    case 7: col_pass<CPB, 7>(src, dst, n, Ns, pin, pout, tw, s); break;
    case 9: col_pass<CPB, 9>(src, dst, n, Ns, pin, pout, tw, s); break;
    default: col_pass<CPB, 8>(src, dst, n, Ns, pin, pout, tw, s); break;
  }
}

}  // namespace

// Column group with the fused middle (plans of at least two passes): the
// forward transform's passes but the last, the fused last-forward x PSF x
// first-inverse pass, the inverse's middle passes (plan I: the same radices
// reversed), and its last pass straight to global memory.  Shared memory
// (cols32_fused_smem): both plans' twiddles and two FFT buffers of
// padded_len(Ly * CPB) elements; the PSF spectrum is read from global memory
// in the fused pass.
template <int MODE, int CPB>
__device__ __forceinline__ void cols_group_fused(unsigned char *smem_raw, cplx<float> *spec, long pitch, int nColsC,
                                                 int nRowsIn, int nRowsOut, const cplx<float> *H, long hPitch,
                                                 const FFTPlan<float> &F, const FFTPlan<float> &I, float scale,
                                                 int c0) {
  const int Ly = F.n;
  const int bufLen = padded_len(Ly * CPB, 2);
  cplx<float> *twF = reinterpret_cast<cplx<float> *>(smem_raw);
  cplx<float> *twI = twF + Ly;
  cplx<float> *bufA = twI + Ly;
  cplx<float> *bufB = bufA + bufLen;
  const int nl = min(CPB, nColsC - c0);
  if (nl <= 0) return;
  const int pairs = (nl + 1) >> 1;
  const int padF = F.padFirst ? 2 : 0, padI = I.padFirst ? 2 : 0;
  spec += c0;
  H += c0;
  for (int t = threadIdx.x; t < Ly; t += blockDim.x) {
    if (t < nRowsIn)
      load_row<CPB>(bufA + (long)t * CPB, spec + (long)t * pitch, pairs);
    else
      zero_row<CPB>(bufA + (long)t * CPB);
  }
  for (int i = threadIdx.x; 2 * i < Ly; i += blockDim.x) {
    cp_async16(twF + 2 * i, F.tw + 2 * i);
    cp_async16(twI + 2 * i, I.tw + 2 * i);
  }
  cp_async_wait_all();
  __syncthreads();
  const int last = F.npass - 1;
  // forward passes 0 .. last-1
  cplx<float> *src = bufA, *dst = bufB;
  const cplx<float> *tw = twF;
  int Ns = 1;
  for (int ps = 0; ps < last; ps++) {
    const int R = (int)((F.radix >> (4 * ps)) & 15ull);
    mid_pass<CPB>(R, src, dst, Ly, Ns, ps == 1 ? padF : 0, ps == 0 ? padF : 0, tw, -1);
    __syncthreads();
    tw += (R - 1) * Ns;
    Ns *= R;
    cplx<float> *t = src;
    src = dst;
    dst = t;
  }
  const int Rm = (int)((F.radix >> (4 * last)) & 15ull);
  fused_mid_r<MODE, CPB>(Rm, src, dst, H, hPitch, nl, Ly, last == 1 ? padF : 0, padI, tw, scale);
  __syncthreads();
  {
    cplx<float> *t = src;
    src = dst;
    dst = t;
  }
  // inverse passes 1 .. last-1 (plan I; its pass 0 was the fused one)
  tw = twI + (Rm - 1);
  Ns = Rm;
  for (int ps = 1; ps < last; ps++) {
    const int R = (int)((I.radix >> (4 * ps)) & 15ull);
    mid_pass<CPB>(R, src, dst, Ly, Ns, ps == 1 ? padI : 0, 0, tw, +1);
    __syncthreads();
    tw += (R - 1) * Ns;
    Ns *= R;
    cplx<float> *t = src;
    src = dst;
    dst = t;
  }
  pdl_trigger();
  const int Rl = (int)((I.radix >> (4 * last)) & 15ull);
  last_to_global_r<CPB>(Rl, src, spec, pitch, Ly, last == 1 ? padI : 0, tw, nRowsOut, nl);
}

namespace {

// Batch entry y uses H + e * hBatch with e = y / hDiv, or hMap[e] when a map
// is given (hBatch 0: one PSF spectrum for every entry).
template <int MODE, int CPB>
__global__ void __launch_bounds__(1024) k_cols32(cplx<float> *__restrict__ spec, long pitch, long batch,
                                                int nColsC, int nRowsIn, int nRowsOut,
                                                const cplx<float> *__restrict__ H, long hPitch, FFTPlan<float> plan,
                                                FFTPlan<float> planI, float scale, long hBatch, int hDiv,
                                                const int *__restrict__ hMap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_wait();
  if (hBatch) {
    const int e = blockIdx.y / hDiv;
    H += (long)(hMap ? hMap[e] : e) * hBatch;
  }
  if (planI.tw)
    cols_group_fused<MODE, CPB>(smem_raw, spec + blockIdx.y * batch, pitch, nColsC, nRowsIn, nRowsOut, H, hPitch,
                                plan, planI, scale, blockIdx.x * CPB);
  else
    cols_group<MODE, CPB>(smem_raw, spec + blockIdx.y * batch, pitch, nColsC, nRowsIn, nRowsOut, H, hPitch, plan,
                          scale, blockIdx.x * CPB);
}

template <int MODE, int CPB>
cudaError_t launch_one(cplx<float> *s, long pitch, long batch, int nColsC, int nRowsIn, int nRowsOut,
                       const cplx<float> *h, long hPitch, const FFTPlan<float> &p, const FFTPlan<float> &pI,
                       float scale, int nBatch, cudaStream_t st, int threads, long hBatch, int hDiv,
                       const int *hMap) {
  auto kern = k_cols32<MODE, CPB>;
  allow_max_smem((const void *)kern);
  const size_t sm = pI.tw ? cols32_fused_smem(p.n, CPB) : cols32_smem(p.n, CPB);
  dim3 grid((nColsC + CPB - 1) / CPB, nBatch);
  return launch_pdl(kern, grid, dim3(threads), sm, st, s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p,
                    pI, scale, hBatch, hDiv, hMap);
}

template <int MODE>
cudaError_t launch_mode(int cpb, cplx<float> *s, long pitch, long batch, int nColsC, int nRowsIn, int nRowsOut,
                        const cplx<float> *h, long hPitch, const FFTPlan<float> &p, const FFTPlan<float> &pI,
                        float scale, int nBatch, cudaStream_t st, int threads, long hBatch, int hDiv,
                        const int *hMap) {
  switch (cpb) {
    case 1: return launch_one<MODE, 1>(s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p, pI, scale, nBatch, st,
                                       threads, hBatch, hDiv, hMap);
    case 2: return launch_one<MODE, 2>(s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p, pI, scale, nBatch, st,
                                       threads, hBatch, hDiv, hMap);
    case 4: return launch_one<MODE, 4>(s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p, pI, scale, nBatch, st,
                                       threads, hBatch, hDiv, hMap);
    default: return launch_one<MODE, 8>(s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p, pI, scale, nBatch,
                                        st, threads, hBatch, hDiv, hMap);
  }
}

}  // namespace

// Column pass of a ragged cutout set: CTA t serves column group g of spectrum
// `line` of the slot that owns t (each cutout its own lengths and pitch).
constexpr int kRagCpb = kRagColsPerCta;
__global__ void __launch_bounds__(256) k_rag_cols(RagArgs r) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_wait();
  const int t = blockIdx.x;
  const int k = rag_slot(r.start, r.K, t);
  const RagEntry &E = r.ent[r.act[k]];
  const int local = t - r.start[k];
  const int line = local / E.colGroups, g = local - line * E.colGroups;
  cplx<float> *spec = r.spec + (r.lines == 1 ? E.specOff : (long)r.lines * E.specOff + (long)line * E.specSize);
  const float scale = 1.f / ((float)E.Lx * (float)E.Ly);
  if (E.colPlanI.tw)
    cols_group_fused<1, kRagCpb>(smem_raw, spec, E.pitch, E.Lx / 2 + 1, E.winRows, E.nDataRows, r.H + E.hOff,
                                 E.pitch, E.colPlan, E.colPlanI, scale, g * kRagCpb);
  else
    cols_group<1, kRagCpb>(smem_raw, spec, E.pitch, E.Lx / 2 + 1, E.winRows, E.nDataRows, r.H + E.hOff, E.pitch,
                           E.colPlan, scale, g * kRagCpb);
}

cudaError_t launch_rag_cols(const RagArgs &r, int total, int maxLy, cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  allow_max_smem((const void *)k_rag_cols);
  const size_t sm = std::max(cols32_smem(maxLy, kRagCpb), cols32_fused_smem(maxLy, kRagCpb));
  return launch_pdl(k_rag_cols, dim3(total), dim3(128), sm, st, r);
}

// the fused form: both plans' twiddles and the two FFT buffers
size_t cols32_fused_smem(int Ly, int cpb) {
  return sizeof(cplx<float>) * (2 * (size_t)Ly + 2 * (size_t)padded_len(Ly * cpb, 2));
}

size_t cols32_smem(int Ly, int cpb) {
  return sizeof(cplx<float>) * ((size_t)Ly * (1 + cpb) + 2 * (size_t)padded_len(Ly * cpb, 2));
}

cudaError_t launch_cols32(void *spec, long pitch, long batch, int nColsC, int nRowsIn, int nRowsOut, const void *H,
                          long hPitch, const FFTLen &Ly, float scale, int mode, int nBatch, cudaStream_t st, int cpb,
                          long hBatch, int hDiv, const int *hMap, int threads) {
  if ((pitch & 1) || (hPitch & 1) || (Ly.full.n & 1) || mode < 1 || mode > 2) return cudaErrorInvalidValue;
  int optin = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (cpb <= 0) cpb = (nColsC * nBatch >= 4 * 152) ? 4 : 2;
  if (cpb != 1 && cpb != 2 && cpb != 4) cpb = 8;
  auto need = [&](int c) { return std::max(cols32_smem(Ly.full.n, c), cols32_fused_smem(Ly.full.n, c)); };
  while (cpb > 1 && need(cpb) > (size_t)optin) cpb >>= 1;
  if (need(cpb) > (size_t)optin) return cudaErrorInvalidValue;
  if (threads <= 0) threads = line_threads(Ly.full.n * cpb / 4);
  FFTPlan<float> p;
  p.n = Ly.full.n;
  p.npass = Ly.full.npass;
  p.radix = pack_radix(Ly.full.radix, Ly.full.npass);
  p.tw = reinterpret_cast<const cplx<float> *>(Ly.full.tw32);
  p.padFirst = fft_pad_enabled() && fft_pad_first(p.npass, p.radix);
  // the inverse half with the radices reversed, for the fused middle pass
  FFTPlan<float> pI{};
  pI.tw = nullptr;
  if (p.npass >= 2 && Ly.fullRev.tw32) {
    pI.n = Ly.fullRev.n;
    pI.npass = Ly.fullRev.npass;
    pI.radix = pack_radix(Ly.fullRev.radix, Ly.fullRev.npass);
    pI.tw = reinterpret_cast<const cplx<float> *>(Ly.fullRev.tw32);
    pI.padFirst = fft_pad_enabled() && fft_pad_first(pI.npass, pI.radix);
  }
  cplx<float> *s = reinterpret_cast<cplx<float> *>(spec);
  const cplx<float> *h = reinterpret_cast<const cplx<float> *>(H);
  if (mode == 1)
    return launch_mode<1>(cpb, s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p, pI, scale, nBatch, st, threads,
                          hBatch, hDiv, hMap);
  return launch_mode<2>(cpb, s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p, pI, scale, nBatch, st, threads,
                        hBatch, hDiv, hMap);
}

void cols32_prepare_kernels() {
  allow_max_smem((const void *)k_cols32<1, 1>);
  allow_max_smem((const void *)k_cols32<1, 2>);
  allow_max_smem((const void *)k_cols32<1, 4>);
  allow_max_smem((const void *)k_cols32<1, 8>);
  allow_max_smem((const void *)k_cols32<2, 1>);
  allow_max_smem((const void *)k_cols32<2, 2>);
  allow_max_smem((const void *)k_cols32<2, 4>);
  allow_max_smem((const void *)k_cols32<2, 8>);
}

}  // namespace imfit
