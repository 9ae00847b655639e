// kernels.h -- host-side launch interface of the GB300 kernels (internal to
// the library; the public C ABI is include/imfit_gb300.h).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "common.cuh"

namespace imfit {

// One FFT length with its radix schedule and device twiddle tables.
struct FFTTable {
  int n = 0;
  int npass = 0;
  int radix[16] = {0};
  void *tw64 = nullptr;  // n complex doubles: exp(-2 pi i k / n)
  void *tw32 = nullptr;  // n complex floats
};

// A padded real line length L (even): the half-length complex transform used
// for rows (M = L/2), the full-length transform used for columns, and the
// split twiddles exp(-2 pi i k / L), k = 0..L/2.
struct FFTLen {
  int L = 0;
  FFTTable half;
  FFTTable full;
  void *twL64 = nullptr;
  void *twL32 = nullptr;
};

// smallest 7-smooth (2,3,5,7) integer >= n, optionally even
int smooth_size(int n, bool even);
// radix schedule (8,4,2,3,5,7 preference); returns number of passes or -1
int radix_schedule(int n, int *radix);
// allocate/free the device tables of one length
cudaError_t fftlen_create(FFTLen &L, int len);
void fftlen_destroy(FFTLen &L);

template <typename T>
cudaError_t launch_rows_r2c(const T *in, long inPitch, long inBatch, int inCols, int nRows, void *out,
                            long outPitch, long outBatch, const FFTLen &Lx, int nBatch, cudaStream_t st);
template <typename T>
cudaError_t launch_cols(void *spec, long pitch, long batch, int nColsC, int nRowsIn, int nRowsOut,
                        const void *H, long hPitch, const FFTLen &Ly, T scale, int mode, int nBatch,
                        cudaStream_t st);
template <typename T>
cudaError_t launch_rows_c2r(const void *in, long inPitch, long inBatch, int nRows, T *out, long outPitch,
                            long outBatch, int outCols, T scale, const FFTLen &Lx, int nBatch,
                            cudaStream_t st);

// ---------------------------------------------------------------- plain FP64
// Model grid description: pixel (i,j) has coordinates
//   main   : x = j - pc + 1,               y = i - pr + 1
//   region : x = x1 + off + (j - pc)*frac, y = y1 + off + (i - pr)*frac
struct Grid64 {
  int nCols, nRows;
  int pc, pr;
  int isRegion;
  int x1, y1;
  double off, frac;
};

cudaError_t launch_eval64(const CompF64 *comps, int nComp, double *model, long pitch, Grid64 g,
                          cudaStream_t st);
cudaError_t launch_downsample64(const double *region, int nOC, int nOR, int osPsfCols, int osPsfRows,
                                double *mainImg, int nMainCols, int nMainRows, int mainPsfCols,
                                int mainPsfRows, int x1, int y1, int scale, cudaStream_t st);

// statistic over the data crop (FP64).  kind: 0 chi^2 (enorm^2), 1 Cash, 2 PMLR-Cash
struct StatArgs64 {
  const double *model;   // model image (crop mapping below)
  const double *data;
  const double *weight;  // internal weights (1/sigma, masked)
  const double *extra;   // extra Cash terms (or null)
  const double *mask;    // for model-error weight updates
  const long *boot;      // bootstrap indices or null
  long nz;               // number of terms (nData or nValid)
  int nDataCols;
  int modelCols, offR, offC;  // model index = modelCols*(offR+row) + offC + col
  double effGain, sky, rnTerm;  // rnTerm = nCombined * readNoise_adu^2
  int modelErrors;
  int kind;
};
cudaError_t launch_deviates64(const StatArgs64 &a, double *dev, double *wOut, cudaStream_t st);
// deterministic two-level reduction; partials must hold >= kStatBlocks * 8 doubles
constexpr int kStatBlocks = 296;
cudaError_t launch_statistic64(const StatArgs64 &a, double *partials, double *result, cudaStream_t st);
// one finite-difference gradient column: out = sum_z dev0_z * (dev1_z - dev0_z) / h  (deterministic)
cudaError_t launch_fd_dot64(const double *dev0, const double *dev1, long n, double invh, double *partials,
                            double *result, cudaStream_t st);
cudaError_t launch_crop64(const double *model, int modelCols, int offR, int offC, int nCols, int nRows,
                          double *out, cudaStream_t st);

// ----------------------------------------------------------------- fast FP32
struct FastGeom {
  int nDataCols, nDataRows;     // N
  int winCols, winRows;         // W = N + P - 1
  int xOrig, yOrig;             // IRAF coordinate of window pixel (0,0)
  int specPitch;                // complex row pitch of the half spectrum (>= Lx/2+1)
  long specBatch;               // complex elements per batch entry
  // oversampled region (nRegion = 0 when absent)
  int hasRegion;
  int rx0, ry0;                 // 0-based data column/row of the region's first replaced pixel
  int rCols, rRows;             // replaced pixels (after the reference's size rule)
  int rScale;
  int rWinCols, rWinRows;       // region window (nSub + Pos - 1)
  int rSubCols, rSubRows;       // subpixels covered by replaced data pixels
  int rXBase, rYBase;           // IRAF integer part of region window pixel (0,0) coordinate
  int rWinOffX, rWinOffY;       // 1 + c_os - P_os per axis: window index -> region subpixel index
  float rStartOff, rFrac;       // 0.5/k - 0.5, 1/k
  int rSpecPitch;
  long rSpecBatch;
};

struct FastArgs {
  // static model description
  const CompDesc *desc;
  int nComp, nParams;
  // per-batch state
  const double *params;  // [B][nParams]
  CompF32 *comps;        // [B][nComp]
  float *bgLevel;        // [B] constant background added after convolution
  // data (FP32 copies) and statistic
  const float *data;     // N
  const float *weight;   // internal weights (masked), or multiplicity-weighted
  const float *extra;    // Cash extra terms (or null)
  const float *count;    // bootstrap multiplicity per pixel (or null)
  int kind;              // 0 chi^2, 1 Cash
  int modelErrors;
  float effGain, sky, rnTerm;
  float psfSum, psfSumOs;
  // spectra and scratch
  void *spec;            // main half spectrum [B][Ly][specPitch] complex float
  void *rspec;           // region half spectrum
  float *regModel;       // [B][rRows][rCols] downsampled region model
  float *regG;           // [B][rRows][rCols] dS/dM for region pixels
  double *statPart;      // [B][nStatBlocks][2]   (S, sum g)
  double *gradPart;      // [B][nGradBlocks][nParams]
  int nStatBlocks, nGradBlocks, nRegGradBlocks;
  double *stat;          // [B]
  double *grad;          // [B][nParams]
  float *modelOut;       // optional: [B][N] model image (FP32) for inspection
};

// Optional per-stage CUDA events: an event is recorded on the launch stream
// after every kernel of the fast path (recorded into the graph when captured).
struct StageTimer {
  static constexpr int kMax = 48;
  cudaEvent_t ev[kMax];
  const char *names[kMax];
  int n = 0;
};

struct FastPlan {
  StageTimer *timer = nullptr;
  FastGeom g;
  const FFTLen *Lx, *Ly, *Rx, *Ry;  // main and region lengths
  const void *H, *Hr;               // FP32 PSF spectra (main, region)
  long hPitch, hrPitch;
};

cudaError_t fast_setup(const FastArgs &a, int nBatch, cudaStream_t st);
cudaError_t fast_forward(const FastPlan &p, const FastArgs &a, int nBatch, bool wantGrad, cudaStream_t st);
cudaError_t fast_adjoint(const FastPlan &p, const FastArgs &a, int nBatch, cudaStream_t st);
int fast_stat_blocks(const FastGeom &g);
int fast_grad_blocks(const FastGeom &g);
int fast_reg_grad_blocks(const FastGeom &g);

}  // namespace imfit
