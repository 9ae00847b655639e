// k_fft.cu -- 2-D real convolution kernels (FP64 plain path and FP32 helpers).
//
// The reference convolves the zero-padded model with the PSF by FFTW r2c,
// complex multiply, c2r and a 1/N rescale (core/convolver.cpp:340-414).  Here
// the 2-D transform is split into
//   1. k_rows_r2c   : each row -> half spectrum (real row packed as M = L/2
//                     complex points, M-point FFT, split), rows beyond the
//                     image are implicit zeros and never read;
//   2. k_cols       : each group of half-spectrum columns -> column FFT,
//                     multiply by the cached PSF spectrum (or its conjugate
//                     for the adjoint), inverse column FFT, all in shared
//                     memory with a single read and write of the spectrum;
//   3. k_rows_c2r   : each needed row -> real row, rescaled.
// Padded lengths are 7-smooth, at least as large as the reference's
// (N + P - 1); linear convolution is unchanged by extra zero padding.
#include "kernels.h"
#include "fft.cuh"

namespace imfit {

template <typename T>
__global__ void __launch_bounds__(1024) k_rows_r2c(const T *__restrict__ in, long inPitch, long inBatch,
                                                  int inCols, int nRows, cplx<T> *__restrict__ out,
                                                  long outPitch, long outBatch, FFTPlan<T> plan,
                                                  const cplx<T> *__restrict__ twL, int rpb) {
  extern __shared__ unsigned char smem_raw[];
  cplx<T> *bufA = reinterpret_cast<cplx<T> *>(smem_raw);
  const int M = plan.n;
  const int ls = M + 1;
  cplx<T> *bufB = bufA + rpb * ls;
  const int row0 = blockIdx.x * rpb;
  const int b = blockIdx.y;
  const int nl = min(rpb, nRows - row0);
  if (nl <= 0) return;
  in += b * inBatch;
  out += b * outBatch;
  const FastDiv byM(M), byM1(M + 1);
  for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
    const int l = byM.div(idx), k = idx - l * M;
    const T *src = in + (long)(row0 + l) * inPitch;
    const int c0 = 2 * k, c1 = 2 * k + 1;
    cplx<T> z;
    z.x = (c0 < inCols) ? src[c0] : (T)0;
    z.y = (c1 < inCols) ? src[c1] : (T)0;
    bufA[l * ls + k] = z;
  }
  __syncthreads();
  cplx<T> *Z = block_fft(bufA, bufB, plan, nl, ls, 1, -1, false);
  for (int idx = threadIdx.x; idx < nl * (M + 1); idx += blockDim.x) {
    const int l = byM1.div(idx), k = idx - l * (M + 1);
    out[(long)(row0 + l) * outPitch + k] = r2c_post(Z + l * ls, k, M, twL);
  }
}

// H of batch entry y is H + e * hBatch with e = y / hDiv, or hMap[e] when a map
// is given (hBatch 0: one PSF for all).
template <typename T, int MODE>
__global__ void __launch_bounds__(1024) k_cols(cplx<T> *__restrict__ spec, long pitch, long batch, int nColsC,
                                              int nRowsIn, int nRowsOut, const cplx<T> *__restrict__ H,
                                              long hPitch, FFTPlan<T> plan, T scale, int cpb, long hBatch,
                                              int hDiv, const int *__restrict__ hMap) {
  extern __shared__ unsigned char smem_raw[];
  cplx<T> *bufA = reinterpret_cast<cplx<T> *>(smem_raw);
  const int Ly = plan.n;
  cplx<T> *bufB = bufA + Ly * cpb;
  const int c0 = blockIdx.x * cpb;
  const int nl = min(cpb, nColsC - c0);
  if (nl <= 0) return;
  const FastDiv byCpb(cpb);
  spec += blockIdx.y * batch;
  if (hBatch) {
    const int e = blockIdx.y / hDiv;
    H += (long)(hMap ? hMap[e] : e) * hBatch;
  }
  for (int idx = threadIdx.x; idx < Ly * cpb; idx += blockDim.x) {
    const int t = byCpb.div(idx), f = idx - t * cpb;
    cplx<T> v = {(T)0, (T)0};
    if (t < nRowsIn && f < nl) v = spec[(long)t * pitch + c0 + f];
    bufA[t * cpb + f] = v;
  }
  __syncthreads();
  cplx<T> *X = block_fft(bufA, bufB, plan, cpb, 1, cpb, -1, true);
  if constexpr (MODE == 0) {
    for (int idx = threadIdx.x; idx < Ly * cpb; idx += blockDim.x) {
      const int t = byCpb.div(idx), f = idx - t * cpb;
      if (f < nl) spec[(long)t * pitch + c0 + f] = X[t * cpb + f];
    }
  } else {
  for (int idx = threadIdx.x; idx < Ly * cpb; idx += blockDim.x) {
    const int t = byCpb.div(idx), f = idx - t * cpb;
    if (f < nl) {
      cplx<T> h = H[(long)t * hPitch + c0 + f];
      if (MODE == 2) h.y = -h.y;
      cplx<T> v = cmul(X[t * cpb + f], h);
      v.x *= scale;
      v.y *= scale;
      X[t * cpb + f] = v;
    }
  }
  __syncthreads();
  cplx<T> *other = (X == bufA) ? bufB : bufA;
  cplx<T> *Y = block_fft(X, other, plan, cpb, 1, cpb, +1, true);
  for (int idx = threadIdx.x; idx < nRowsOut * cpb; idx += blockDim.x) {
    const int t = byCpb.div(idx), f = idx - t * cpb;
    if (f < nl) spec[(long)t * pitch + c0 + f] = Y[t * cpb + f];
  }
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) k_rows_c2r(const cplx<T> *__restrict__ in, long inPitch, long inBatch,
                                                  int nRows, T *__restrict__ out, long outPitch,
                                                  long outBatch, int outCols, T scale, FFTPlan<T> plan,
                                                  const cplx<T> *__restrict__ twL, int rpb) {
  extern __shared__ unsigned char smem_raw[];
  const int M = plan.n;
  const int ls = M + 1;
  cplx<T> *bufX = reinterpret_cast<cplx<T> *>(smem_raw);
  cplx<T> *bufA = bufX + rpb * ls;
  cplx<T> *bufB = bufA + rpb * ls;
  const int row0 = blockIdx.x * rpb;
  const int nl = min(rpb, nRows - row0);
  if (nl <= 0) return;
  in += blockIdx.y * inBatch;
  out += blockIdx.y * outBatch;
  const FastDiv byM(M), byM1(M + 1), byOut(outCols);
  for (int idx = threadIdx.x; idx < nl * (M + 1); idx += blockDim.x) {
    const int l = byM1.div(idx), k = idx - l * (M + 1);
    bufX[l * ls + k] = in[(long)(row0 + l) * inPitch + k];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < nl * M; idx += blockDim.x) {
    const int l = byM.div(idx), k = idx - l * M;
    bufA[l * ls + k] = c2r_pre(bufX + l * ls, k, M, twL);
  }
  __syncthreads();
  cplx<T> *Z = block_fft(bufA, bufB, plan, nl, ls, 1, +1, false);
  for (int idx = threadIdx.x; idx < nl * outCols; idx += blockDim.x) {
    const int l = byOut.div(idx), c = idx - l * outCols;
    const cplx<T> z = Z[l * ls + (c >> 1)];
    out[(long)(row0 + l) * outPitch + c] = scale * ((c & 1) ? z.y : z.x);
  }
}

// ------------------------------------------------------------------ launchers
template <typename T>
static FFTPlan<T> plan_of(const FFTLen &L, bool half) {
  FFTPlan<T> p;
  const FFTTable &t = half ? L.half : L.full;
  p.n = t.n;
  p.npass = t.npass;
  p.radix = pack_radix(t.radix, t.npass);
  p.tw = reinterpret_cast<const cplx<T> *>(sizeof(T) == 8 ? (const void *)t.tw64 : (const void *)t.tw32);
  return p;
}

template <typename T>
static const cplx<T> *twl_of(const FFTLen &L) {
  return reinterpret_cast<const cplx<T> *>(sizeof(T) == 8 ? (const void *)L.twL64 : (const void *)L.twL32);
}

// One line per CTA and about one thread per complex point: the FFT passes of a
// line then have one butterfly per thread, and many small CTAs keep the SMs
// occupied even for a single image.
int rows_per_block(int M, int elemBytes, int nbuf) {
  (void)M;
  (void)elemBytes;
  (void)nbuf;
  return 1;
}

int line_threads(int points) {
  int t = (points + 31) / 32 * 32;
  if (t < 64) t = 64;
  if (t > 1024) t = 1024;
  return t;
}

template <typename T>
cudaError_t launch_rows_r2c(const T *in, long inPitch, long inBatch, int inCols, int nRows, void *out,
                            long outPitch, long outBatch, const FFTLen &Lx, int nBatch, cudaStream_t st) {
  const int M = Lx.half.n;
  const int rpb = rows_per_block(M, sizeof(T), 2);
  const size_t sm = sizeof(cplx<T>) * 2 * (size_t)rpb * (M + 1);
  auto kern = k_rows_r2c<T>;
  allow_max_smem((const void *)kern);
  dim3 grid((nRows + rpb - 1) / rpb, nBatch);
  kern<<<grid, line_threads(M * rpb), sm, st>>>(in, inPitch, inBatch, inCols, nRows, reinterpret_cast<cplx<T> *>(out), outPitch,
                              outBatch, plan_of<T>(Lx, true), twl_of<T>(Lx), rpb);
  return cudaGetLastError();
}

int cols_per_block(int Ly, int elemBytes, int nColsC) {
  // two ping-pong buffers of Ly x cpb complex per CTA; one or two columns per
  // CTA, two only when that still leaves several CTAs per SM
  int cpb = (nColsC >= 600) ? 2 : 1;
  while (cpb > 1 && (size_t)2 * Ly * cpb * 2 * elemBytes > 200 * 1024) cpb >>= 1;
  return cpb;
}

template <typename T>
cudaError_t launch_cols(void *spec, long pitch, long batch, int nColsC, int nRowsIn, int nRowsOut,
                        const void *H, long hPitch, const FFTLen &Ly, T scale, int mode, int nBatch,
                        cudaStream_t st, int cpbOverride, long hBatch, int hDiv, const int *hMap,
                        int threadsOverride) {
  const int L = Ly.full.n;
  int cpb = cpbOverride > 0 ? cpbOverride : cols_per_block(L, sizeof(T), nColsC);
  while (cpb > 1 && (size_t)2 * L * cpb * 2 * sizeof(T) > 200 * 1024) cpb >>= 1;
  const size_t sm = sizeof(cplx<T>) * 2 * (size_t)L * cpb;
  dim3 grid((nColsC + cpb - 1) / cpb, nBatch);
  const int nt = threadsOverride > 0 ? threadsOverride : line_threads(L * cpb / 2);
  auto p = plan_of<T>(Ly, false);
  cplx<T> *s = reinterpret_cast<cplx<T> *>(spec);
  const cplx<T> *h = reinterpret_cast<const cplx<T> *>(H);
  if (mode == 0) {
    allow_max_smem((const void *)k_cols<T, 0>);
    k_cols<T, 0><<<grid, nt, sm, st>>>(s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p, scale, cpb, hBatch, hDiv, hMap);
  } else if (mode == 1) {
    allow_max_smem((const void *)k_cols<T, 1>);
    k_cols<T, 1><<<grid, nt, sm, st>>>(s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p, scale, cpb, hBatch, hDiv, hMap);
  } else {
    allow_max_smem((const void *)k_cols<T, 2>);
    k_cols<T, 2><<<grid, nt, sm, st>>>(s, pitch, batch, nColsC, nRowsIn, nRowsOut, h, hPitch, p, scale, cpb, hBatch, hDiv, hMap);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_rows_c2r(const void *in, long inPitch, long inBatch, int nRows, T *out, long outPitch,
                            long outBatch, int outCols, T scale, const FFTLen &Lx, int nBatch,
                            cudaStream_t st) {
  const int M = Lx.half.n;
  const int rpb = rows_per_block(M, sizeof(T), 3);
  const size_t sm = sizeof(cplx<T>) * 3 * (size_t)rpb * (M + 1);
  auto kern = k_rows_c2r<T>;
  allow_max_smem((const void *)kern);
  dim3 grid((nRows + rpb - 1) / rpb, nBatch);
  kern<<<grid, line_threads(M * rpb), sm, st>>>(reinterpret_cast<const cplx<T> *>(in), inPitch, inBatch, nRows, out, outPitch,
                              outBatch, outCols, scale, plan_of<T>(Lx, true), twl_of<T>(Lx), rpb);
  return cudaGetLastError();
}

template cudaError_t launch_rows_r2c<double>(const double *, long, long, int, int, void *, long, long,
                                             const FFTLen &, int, cudaStream_t);
template cudaError_t launch_rows_r2c<float>(const float *, long, long, int, int, void *, long, long,
                                            const FFTLen &, int, cudaStream_t);
template cudaError_t launch_cols<double>(void *, long, long, int, int, int, const void *, long,
                                         const FFTLen &, double, int, int, cudaStream_t, int, long, int, const int *, int);
template cudaError_t launch_cols<float>(void *, long, long, int, int, int, const void *, long,
                                        const FFTLen &, float, int, int, cudaStream_t, int, long, int, const int *, int);
template cudaError_t launch_rows_c2r<double>(const void *, long, long, int, double *, long, long, int,
                                             double, const FFTLen &, int, cudaStream_t);
template cudaError_t launch_rows_c2r<float>(const void *, long, long, int, float *, long, long, int, float,
                                            const FFTLen &, int, cudaStream_t);

}  // namespace imfit

// ------------------------------------------------------------ FFT tables
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <set>
#include <utility>
#include <vector>

namespace imfit {

void fft_prepare_kernels() {
  allow_max_smem((const void *)k_rows_r2c<float>);
  allow_max_smem((const void *)k_rows_r2c<double>);
  allow_max_smem((const void *)k_rows_c2r<float>);
  allow_max_smem((const void *)k_rows_c2r<double>);
  allow_max_smem((const void *)k_cols<float, 0>);
  allow_max_smem((const void *)k_cols<float, 1>);
  allow_max_smem((const void *)k_cols<float, 2>);
  allow_max_smem((const void *)k_cols<double, 0>);
  allow_max_smem((const void *)k_cols<double, 1>);
  allow_max_smem((const void *)k_cols<double, 2>);
}

bool pdl_enabled() {
  static const bool on = [] {
    const char *v = getenv("IMFIT_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}

// Padded first intermediate of the column FFTs (fft_pad_first); IMFIT_FFT_PAD=0
// keeps every layout unpadded.
bool fft_pad_enabled() {
  static const bool on = [] {
    const char *v = getenv("IMFIT_FFT_PAD");
    return !(v && v[0] == '0');
  }();
  return on;
}

void allow_max_smem(const void *kernel) {
  static std::mutex lock;
  static std::set<std::pair<int, const void *>> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> g(lock);
  if (!done.insert({dev, kernel}).second) return;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return;
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}

static bool is_smooth(int n) {
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}

int smooth_size(int n, bool even) {
  if (n < 2) n = 2;
  for (int m = n;; m++) {
    if (even && (m & 1)) continue;
    if (is_smooth(m)) return m;
  }
}

// Radix orders the fast path's autotuner chooses among (the transform is the
// same; the pass count, the work per pass and the twiddle traffic differ);
// each takes the listed radices greedily, as often as they divide:
//   0: 8, 9, 4, 2, then 3, 5, 7;
//   1: the odd radices 7, 5, 9, 3 first, then 8, 4, 2;
//   2: 4 and 2 instead of 8, then 9, 3, 5, 7;
//   kRadixPlain (the FP64 drop-in's plans): 8, 4, 2, 3, 5, 7 (no radix 9,
//   whose 3 x 3 butterfly rounds differently from two radix-3 passes).
int radix_schedule(int n, int *radix, int variant) {
  int np = 0;
  auto take = [&](int p) {
    while (n % p == 0 && np < kMaxRadixPasses) {
      radix[np++] = p;
      n /= p;
    }
  };
  if (variant == kRadixPlain) {
    for (int p : {8, 4, 2, 3, 5, 7}) take(p);
  } else if (variant == 1) {
    for (int p : {7, 5, 9, 3, 8, 4, 2}) take(p);
  } else if (variant == 2) {
    for (int p : {4, 2, 9, 3, 5, 7}) take(p);
  } else {
    for (int p : {8, 9, 4, 2, 3, 5, 7}) take(p);
  }
  return (n == 1) ? np : -1;
}

// The `count` smallest 7-smooth lengths >= n (even if asked) within
// maxRatio * n (the smallest one always).
int smooth_candidates(int n, bool even, int count, double maxRatio, int *out) {
  int k = 0;
  for (int m = smooth_size(n, even); k < count; m = smooth_size(m + 1, even)) {
    if (k > 0 && m > maxRatio * n) break;
    out[k++] = m;
  }
  return k;
}

// Twiddles of the plan, pass by pass: pass p (radix R, span Ns, starting at
// offset off_p = sum over earlier passes of (R_q - 1) Ns_q) holds
// exp(-2 pi i r k / (Ns R)) at off_p + (r - 1) Ns + k, r in [1, R), k in
// [0, Ns) -- n - 1 entries in all.  Threads of a pass with consecutive k then
// read consecutive entries (no shared-memory bank conflicts once staged);
// each value is the one a single table exp(-2 pi i m / n) holds at
// m = r k n / (Ns R).
static cudaError_t table_create(FFTTable &t, int n, int variant, bool reversed = false) {
  t.n = n;
  t.npass = radix_schedule(n, t.radix, variant);
  if (t.npass < 0) return cudaErrorInvalidValue;
  if (reversed)
    for (int i = 0, j = t.npass - 1; i < j; i++, j--) std::swap(t.radix[i], t.radix[j]);
  std::vector<double> full(2 * (size_t)n);
  for (int k = 0; k < n; k++) {
    const double a = 2.0 * M_PI * (double)k / (double)n;
    full[2 * k] = cos(a);
    full[2 * k + 1] = -sin(a);
  }
  std::vector<double> w64(2 * (size_t)n, 0.0);
  std::vector<float> w32(2 * (size_t)n, 0.f);
  long off = 0;
  for (int p = 0, Ns = 1; p < t.npass; Ns *= t.radix[p], p++) {
    const int R = t.radix[p], step = n / (Ns * R);
    for (int r = 1; r < R; r++)
      for (int k = 0; k < Ns; k++) {
        const long e = off + (long)(r - 1) * Ns + k, m = (long)r * k * step;
        w64[2 * e] = full[2 * m];
        w64[2 * e + 1] = full[2 * m + 1];
      }
    off += (long)(R - 1) * Ns;
  }
  for (size_t i = 0; i < w64.size(); i++) w32[i] = (float)w64[i];
  cudaError_t e = cudaMalloc(&t.tw64, sizeof(double) * 2 * (size_t)n);
  if (e) return e;
  e = cudaMalloc(&t.tw32, sizeof(float) * 2 * (size_t)n);
  if (e) return e;
  e = cudaMemcpy(t.tw64, w64.data(), sizeof(double) * 2 * (size_t)n, cudaMemcpyHostToDevice);
  if (e) return e;
  return cudaMemcpy(t.tw32, w32.data(), sizeof(float) * 2 * (size_t)n, cudaMemcpyHostToDevice);
}

cudaError_t fftlen_create(FFTLen &L, int len, int variant) {
  L.L = len;
  L.variant = variant;
  cudaError_t e = table_create(L.full, len, variant);
  if (e) return e;
  e = table_create(L.fullRev, len, variant, true);
  if (e) return e;
  if (len % 2 == 0) {
    e = table_create(L.half, len / 2, variant);
    if (e) return e;
    const int M = len / 2;
    std::vector<double> w64(2 * (size_t)(M + 1));
    std::vector<float> w32(2 * (size_t)(M + 1));
    for (int k = 0; k <= M; k++) {
      const double a = 2.0 * M_PI * (double)k / (double)len;
      w64[2 * k] = cos(a);
      w64[2 * k + 1] = -sin(a);
      w32[2 * k] = (float)w64[2 * k];
      w32[2 * k + 1] = (float)w64[2 * k + 1];
    }
    e = cudaMalloc(&L.twL64, sizeof(double) * 2 * (size_t)(M + 1));
    if (e) return e;
    e = cudaMalloc(&L.twL32, sizeof(float) * 2 * (size_t)(M + 1));
    if (e) return e;
    e = cudaMemcpy(L.twL64, w64.data(), sizeof(double) * 2 * (size_t)(M + 1), cudaMemcpyHostToDevice);
    if (e) return e;
    e = cudaMemcpy(L.twL32, w32.data(), sizeof(float) * 2 * (size_t)(M + 1), cudaMemcpyHostToDevice);
  }
  return e;
}

static void table_destroy(FFTTable &t) {
  if (t.tw64) cudaFree(t.tw64);
  if (t.tw32) cudaFree(t.tw32);
  t.tw64 = t.tw32 = nullptr;
}

void fftlen_destroy(FFTLen &L) {
  table_destroy(L.full);
  table_destroy(L.fullRev);
  table_destroy(L.half);
  if (L.twL64) cudaFree(L.twL64);
  if (L.twL32) cudaFree(L.twL32);
  L.twL64 = L.twL32 = nullptr;
}

}  // namespace imfit
