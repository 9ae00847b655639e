// fft.cuh -- shared-memory mixed-radix Stockham FFT for the PSF convolution.
//
// Replaces the reference's FFTW r2c/c2r convolution (core/convolver.cpp:340-414).
// A CTA transforms several independent lines (rows of the model window, or
// columns of the half spectrum) held in shared memory.  Each pass of radix R
// with span Ns reads src[j + r*n/R], multiplies by exp(s*2*pi*i*r*(j mod Ns)/(Ns*R)),
// performs a length-R DFT in registers and writes dst[(j/Ns)*Ns*R + (j mod Ns) + t*Ns]
// (the self-sorting Stockham formulation), so no bit reversal is needed and
// the output is in natural order after the last pass.  Lengths are products
// of 2, 3, 4, 5, 7, 8 and 9; padded sizes are always chosen from that set.
#pragma once
#include <cuda_runtime.h>

namespace imfit {

template <typename T>
struct cplx {
  T x, y;
};

template <typename T>
__device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T>
__device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T>
__device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) { return {a.x - b.x, a.y - b.y}; }
// multiply by s*i (s = +1 or -1)
template <typename T>
__device__ __forceinline__ cplx<T> mul_si(cplx<T> a, int s) { return s > 0 ? cplx<T>{-a.y, a.x} : cplx<T>{a.y, -a.x}; }

constexpr int kMaxRadixPasses = 16;

// Plan of one transform length: radices applied in order (4 bits each,
// first pass in the low bits: a scalar, so kernels keep the plan in
// registers instead of indexing an array in local memory), plus the twiddle
// table, pass by pass: pass p (radix R, span Ns) holds exp(-2*pi*i*r*k/(Ns*R))
// at off_p + (r-1)*Ns + k (r in [1,R), k in [0,Ns), off_p the sum of
// (R_q - 1) * Ns_q over the earlier passes); n entries allocated.
template <typename T>
struct FFTPlan {
  int n;
  int npass;
  unsigned long long radix;
  const cplx<T> *tw;
  int padFirst = 0;  // kernels that support it: first intermediate in the padded layout (fft_pad_first)
};

inline unsigned long long pack_radix(const int *radix, int npass) {
  unsigned long long r = 0;
  for (int i = 0; i < npass && i < kMaxRadixPasses; i++) r |= (unsigned long long)(radix[i] & 15) << (4 * i);
  return r;
}

// length-R DFT in registers, sign s (-1 forward, +1 inverse)
template <typename T>
__device__ __forceinline__ void dft2(cplx<T> *v) {
  cplx<T> a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <typename T>
__device__ __forceinline__ void dft3(cplx<T> *v, int s) {
  const T h = (T)0.86602540378443864676;
  cplx<T> t1 = cadd(v[1], v[2]);
  cplx<T> t2 = {v[0].x - (T)0.5 * t1.x, v[0].y - (T)0.5 * t1.y};
  cplx<T> d = csub(v[1], v[2]);
  cplx<T> t3 = mul_si(cplx<T>{h * d.x, h * d.y}, s);
  v[0] = cadd(v[0], t1);
  v[1] = cadd(t2, t3);
  v[2] = csub(t2, t3);
}

template <typename T>
__device__ __forceinline__ void dft4(cplx<T> *v, int s) {
  cplx<T> a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
  cplx<T> a2 = cadd(v[1], v[3]), d = csub(v[1], v[3]);
  cplx<T> e = mul_si(d, s);
  v[0] = cadd(a0, a2);
  v[2] = csub(a0, a2);
  v[1] = cadd(a1, e);
  v[3] = csub(a1, e);
}

template <typename T>
__device__ __forceinline__ void dft5(cplx<T> *v, int s) {
  const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
  const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
  cplx<T> a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
  cplx<T> a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
  cplx<T> r1 = {v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y};
  cplx<T> r2 = {v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y};
  cplx<T> i1 = mul_si(cplx<T>{s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y}, s);
  cplx<T> i2 = mul_si(cplx<T>{s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y}, s);
  v[0] = {v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y};
  v[1] = cadd(r1, i1);
  v[4] = csub(r1, i1);
  v[2] = cadd(r2, i2);
  v[3] = csub(r2, i2);
}

template <typename T>
__device__ __forceinline__ void dft7(cplx<T> *v, int s) {
  const T C[3] = {(T)0.62348980185873353053, (T)-0.22252093395631440429, (T)-0.90096886790241912624};
  const T S[3] = {(T)0.78183148246802980871, (T)0.97492791218182360702, (T)0.43388373911755812048};
  cplx<T> a[3], b[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    a[k] = cadd(v[k + 1], v[6 - k]);
    b[k] = csub(v[k + 1], v[6 - k]);
  }
  cplx<T> v0 = v[0];
  v[0] = {v0.x + a[0].x + a[1].x + a[2].x, v0.y + a[0].y + a[1].y + a[2].y};
#pragma unroll
  for (int t = 1; t <= 3; t++) {
    cplx<T> re = v0, im = {0, 0};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int m = ((k + 1) * t) % 7;  // angle index (k+1)*t mod 7
      const T c = (m <= 3) ? C[m - 1] : C[7 - m - 1];
      const T sn = (m <= 3) ? S[m - 1] : -S[7 - m - 1];
      re.x += c * a[k].x;
      re.y += c * a[k].y;
      im.x += sn * b[k].x;
      im.y += sn * b[k].y;
    }
    cplx<T> ii = mul_si(im, s);
    v[t] = cadd(re, ii);
    v[7 - t] = csub(re, ii);
  }
}

template <typename T>
__device__ __forceinline__ void dft8(cplx<T> *v, int s) {
  const T r = (T)0.70710678118654752440;
  cplx<T> e[4] = {v[0], v[2], v[4], v[6]};
  cplx<T> o[4] = {v[1], v[3], v[5], v[7]};
  dft4(e, s);
  dft4(o, s);
  // twiddles W8^k = exp(s*2*pi*i*k/8)
  cplx<T> o1 = {r * (o[1].x - s * o[1].y), r * (o[1].y + s * o[1].x)};
  cplx<T> o2 = mul_si(o[2], s);
  cplx<T> o3 = {r * (-o[3].x - s * o[3].y), r * (-o[3].y + s * o[3].x)};
  v[0] = cadd(e[0], o[0]);
  v[4] = csub(e[0], o[0]);
  v[1] = cadd(e[1], o1);
  v[5] = csub(e[1], o1);
  v[2] = cadd(e[2], o2);
  v[6] = csub(e[2], o2);
  v[3] = cadd(e[3], o3);
  v[7] = csub(e[3], o3);
}

// length-9 DFT as 3 x 3 (Cooley-Tukey, n = n1 + 3 n2, k = k2 + 3 k1): length-3
// DFTs over n2, twiddles W9^(n1 k2) with W9 = exp(s 2 pi i / 9), length-3 DFTs
// over n1; cos / sin of 2 pi e / 9 for e = 1, 2, 4.
template <typename T>
__device__ __forceinline__ void dft9(cplx<T> *v, int s) {
  const T c1 = (T)0.766044443118978035202, s1 = (T)0.642787609686539326323;
  const T c2 = (T)0.173648177666930348852, s2 = (T)0.984807753012208059367;
  const T c4 = (T)-0.939692620785908384054, s4 = (T)0.342020143325668733044;
  cplx<T> y[3][3];
#pragma unroll
  for (int n1 = 0; n1 < 3; n1++) {
    cplx<T> a[3] = {v[n1], v[n1 + 3], v[n1 + 6]};
    dft3(a, s);
    y[n1][0] = a[0];
    y[n1][1] = a[1];
    y[n1][2] = a[2];
  }
  const T sg = (T)s;
  y[1][1] = cmul(y[1][1], cplx<T>{c1, sg * s1});
  y[1][2] = cmul(y[1][2], cplx<T>{c2, sg * s2});
  y[2][1] = cmul(y[2][1], cplx<T>{c2, sg * s2});
  y[2][2] = cmul(y[2][2], cplx<T>{c4, sg * s4});
#pragma unroll
  for (int k2 = 0; k2 < 3; k2++) {
    cplx<T> b[3] = {y[0][k2], y[1][k2], y[2][k2]};
    dft3(b, s);
    v[k2] = b[0];
    v[k2 + 3] = b[1];
    v[k2 + 6] = b[2];
  }
}

// Twiddle exp(s*2*pi*i*idx/n) from the forward table.
template <typename T>
__device__ __forceinline__ cplx<T> twiddle(const cplx<T> *tw, int idx, int s) {
  cplx<T> w = tw[idx];
  if (s > 0) w.y = -w.y;
  return w;
}

// Division by a divisor fixed for a loop, for 0 <= x < 2^21 and d >= 1:
// q = floor((x + 0.5) * (1/d)) with the SFU reciprocal.  (x + 0.5) / d lies
// at least 0.5/d away from every integer, and the computed product is within
// 1.5 * 2^-23 relative of it (reciprocal within 1 ulp, one rounded multiply),
// an error below that margin while x < 2^21.  Every index divided here is
// below 2^16.  Replaces a 32-bit integer division (about twenty
// instructions) by four, and its set-up by one.
struct FastDiv {
  float inv;
  int d;
  __device__ __forceinline__ explicit FastDiv(int dd) : d(dd) {
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"((float)dd));
  }
  __device__ __forceinline__ int div(int x) const { return (int)(((float)x + 0.5f) * inv); }
};

// Shared-memory index with PAD extra elements after every 16: a radix-R first
// pass writes each thread's R outputs at consecutive indices, so lanes store
// R * (lines interleaved) elements apart and, for R = 4 or 8, up to eight
// lanes of a half-warp hit the same banks; two pad elements per 16 spread
// them.  Groups of 16 aligned elements stay contiguous (and 16-byte aligned
// when they start at an even index).
template <int PAD>
__device__ __forceinline__ int pad_idx(int i) {
  return PAD ? i + PAD * (i >> 4) : i;
}

// Elements a buffer of n unpadded elements occupies in the padded layout.
__host__ __device__ inline int padded_len(int n, int pad) { return n + pad * (n >> 4) + pad; }

// Plans whose first pass is radix 4 or 8 (and that have a second pass) write
// their first intermediate in the padded layout.
__host__ __device__ inline bool fft_pad_first(int npass, unsigned long long radix) {
  const int r0 = (int)(radix & 15ull);
  return npass >= 2 && (r0 == 4 || r0 == 8);
}

// One radix-R Stockham pass over 'nl' lines of length n.
// Element t of line l lives at buf[l*ls + t*es] (PIN / POUT: the padding of
// the source / destination layout); tw is this pass's part of the plan's
// twiddle table.
template <typename T, int R, int PIN = 0, int POUT = 0>
__device__ __forceinline__ void stockham_pass(const cplx<T> *__restrict__ src, cplx<T> *__restrict__ dst,
                                              int n, int Ns, int nl, int ls, int es,
                                              const cplx<T> *__restrict__ tw, int s, bool lineFastest) {
  const int m = n / R;
  const int total = m * nl;
  const FastDiv byNl(nl), byM(m), byNs(Ns);
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int l, j;
    if (lineFastest) {
      j = byNl.div(idx);
      l = idx - j * nl;
    } else {
      l = byM.div(idx);
      j = idx - l * m;
    }
    const int k = j - byNs.div(j) * Ns;
    cplx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = src[pad_idx<PIN>(l * ls + (j + r * m) * es)];
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], twiddle(tw, (r - 1) * Ns + k, s));
    }
    if (R == 2) dft2(v);
    if (R == 3) dft3(v, s);
    if (R == 4) dft4(v, s);
    if (R == 5) dft5(v, s);
    if (R == 7) dft7(v, s);
    if (R == 8) dft8(v, s);
    if (R == 9) dft9(v, s);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int t = 0; t < R; t++) dst[pad_idx<POUT>(l * ls + (base + t * Ns) * es)] = v[t];
  }
}

template <typename T, int PIN, int POUT>
__device__ __forceinline__ void radix_pass(int R, const cplx<T> *src, cplx<T> *dst, int n, int Ns, int nl, int ls,
                                           int es, const cplx<T> *tw, int s, bool lineFastest) {
  switch (R) {
    case 2: stockham_pass<T, 2, PIN, POUT>(src, dst, n, Ns, nl, ls, es, tw, s, lineFastest); break;
    case 3: stockham_pass<T, 3, PIN, POUT>(src, dst, n, Ns, nl, ls, es, tw, s, lineFastest); break;
    case 4: stockham_pass<T, 4, PIN, POUT>(src, dst, n, Ns, nl, ls, es, tw, s, lineFastest); break;
    case 5: stockham_pass<T, 5, PIN, POUT>(src, dst, n, Ns, nl, ls, es, tw, s, lineFastest); break;
    case 7: stockham_pass<T, 7, PIN, POUT>(src, dst, n, Ns, nl, ls, es, tw, s, lineFastest); break;
    case 9: stockham_pass<T, 9, PIN, POUT>(src, dst, n, Ns, nl, ls, es, tw, s, lineFastest); break;
    default: stockham_pass<T, 8, PIN, POUT>(src, dst, n, Ns, nl, ls, es, tw, s, lineFastest); break;
  }
}

// Full transform of nl lines; ping-pongs between a and b.  Returns the buffer
// that holds the result.  Must be called by all threads of the CTA.
// tw: the twiddle table to read (null: the plan's own, in global memory;
// kernels that stage the table in shared memory pass their copy).
// PADFIRST: the intermediate written by the first pass (and read by the
// second) uses the padded layout, so both buffers must hold
// padded_len(nl * ls, 2) elements; input and result are unpadded.  Only for
// plans of at least two passes.
template <typename T, bool PADFIRST = false>
__device__ cplx<T> *block_fft(cplx<T> *a, cplx<T> *b, const FFTPlan<T> &p, int nl, int ls, int es,
                              int s, bool lineFastest, const cplx<T> *tw = nullptr) {
  int Ns = 1;
  cplx<T> *src = a, *dst = b;
  if (!tw) tw = p.tw;
  for (int ps = 0; ps < p.npass; ps++) {
    const int R = (int)((p.radix >> (4 * ps)) & 15ull);
    if (PADFIRST && ps == 0)
      radix_pass<T, 0, 2>(R, src, dst, p.n, Ns, nl, ls, es, tw, s, lineFastest);
    else if (PADFIRST && ps == 1)
      radix_pass<T, 2, 0>(R, src, dst, p.n, Ns, nl, ls, es, tw, s, lineFastest);
    else
      radix_pass<T, 0, 0>(R, src, dst, p.n, Ns, nl, ls, es, tw, s, lineFastest);
    __syncthreads();
    tw += (R - 1) * Ns;
    Ns *= R;
    cplx<T> *t = src;
    src = dst;
    dst = t;
  }
  return src;
}

// ---------------------------------------------------------------------------
// Real <-> half-complex helpers for a real line of even length L = 2M packed
// as z[k] = x[2k] + i x[2k+1] (M-point complex FFT).
//   forward:  X[k] = E[k] + W^k O[k],  E = (Z[k] + conj Z[M-k])/2,
//             O = (Z[k] - conj Z[M-k])/(2i),  W = exp(-2 pi i / L),  k = 0..M
//   inverse:  Z[k] = (X[k] + conj X[M-k]) + i W^-k (X[k] - conj X[M-k]),
//             k = 0..M-1; an M-point inverse FFT then yields L*(x[2k] + i x[2k+1]).
// twL[k] = exp(-2*pi*i*k/L) for k in [0, M].

template <typename T>
__device__ __forceinline__ cplx<T> r2c_post(const cplx<T> *Z, int k, int M, const cplx<T> *twL) {
  cplx<T> zk = Z[k == M ? 0 : k];
  cplx<T> zc = Z[k == 0 ? 0 : M - k];
  zc.y = -zc.y;  // conj Z[M-k]
  cplx<T> E = {(T)0.5 * (zk.x + zc.x), (T)0.5 * (zk.y + zc.y)};
  // O = (zk - zc) / (2i) = ( (zk-zc).y/2 , -(zk-zc).x/2 )
  cplx<T> d = csub(zk, zc);
  cplx<T> O = {(T)0.5 * d.y, (T)-0.5 * d.x};
  return cadd(E, cmul(twL[k], O));
}

template <typename T>
__device__ __forceinline__ cplx<T> c2r_pre(const cplx<T> *X, int k, int M, const cplx<T> *twL) {
  cplx<T> xk = X[k];
  cplx<T> xc = X[M - k];
  if (k == 0) { xk.y = 0; xc.y = 0; }  // c2r ignores imag parts of DC / Nyquist
  xc.y = -xc.y;
  cplx<T> E = cadd(xk, xc);
  cplx<T> w = twL[k];
  w.y = -w.y;  // W^-k
  cplx<T> O = cmul(w, csub(xk, xc));
  return {E.x - O.y, E.y + O.x};  // E + i O
}

}  // namespace imfit
