// kernels.h -- host-side launch interface of the GB300 kernels (internal to
// the library; the public C ABI is include/imfit_gb300.h).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <utility>
#include "common.cuh"
#include "fft.cuh"
#include "psf_interp.cuh"

namespace imfit {

// ---------------------------------------------------------------------------
// Programmatic dependent launch (PDL) for the fast path's chain of kernels.
// Each kernel is launched with programmatic stream serialization, so the next
// kernel of the stream (or graph) is scheduled while this one drains; every
// such kernel waits (griddepcontrol.wait) for its predecessor's completion and
// memory before it reads anything the predecessor wrote, and signals
// (griddepcontrol.launch_dependents) once its main work is issued.  The wait is
// the hardware dependency of the launch, not a spin loop.  IMFIT_PDL=0 in the
// environment launches plainly (the waits then return at once).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" :::); }

bool pdl_enabled();
bool fft_pad_enabled();

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  unsigned n = 0;
  if (pdl_enabled()) {
    attr[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[n].val.programmaticStreamSerializationAllowed = 1;
    n++;
  }
  // the stream's priority, explicitly, so that a graph captured from it keeps it
  int prio = 0;
  if (cudaStreamGetPriority(st, &prio) == cudaSuccess && prio != 0) {
    attr[n].id = cudaLaunchAttributePriority;
    attr[n].val.priority = prio;
    n++;
  }
  cfg.attrs = attr;
  cfg.numAttrs = n;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Raise a kernel's dynamic shared-memory limit to the device's opt-in maximum,
// once per (device, kernel).  The limit is never lowered, so launches of one
// kernel with different shared-memory sizes (possibly captured in one graph)
// are all valid.
void allow_max_smem(const void *kernel);

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
  int variant = 0;  // radix order (radix_schedule)
  FFTTable half;
  FFTTable full;
  FFTTable fullRev;  // full length, radices in reverse order (the column pass's inverse half)
  void *twL64 = nullptr;
  void *twL32 = nullptr;
};

// threads of a CTA that transforms lines totalling `points` complex values
int line_threads(int points);
// smallest 7-smooth (2,3,5,7) integer >= n, optionally even
int smooth_size(int n, bool even);

// radix schedule of order `variant` (0: 8,9,4,2,3,5,7; 1: 7,5,9,3,8,4,2;
// 2: 4,2,9,3,5,7; kRadixPlain: 8,4,2,3,5,7); returns the number of passes or -1
int radix_schedule(int n, int *radix, int variant = 0);
constexpr int kRadixVariants = 3;
// the `count` smallest 7-smooth lengths >= n within maxRatio * n; returns how many
int smooth_candidates(int n, bool even, int count, double maxRatio, int *out);
// allocate/free the device tables of one length
// Radix order of the plain FP64 path: 8, 4, 2, 3, 5, 7 (no radix-9 butterflies,
// so its FFT rounding stays that of the validated drop-in); the fast path's
// orders are 0..kRadixVariants-1.
constexpr int kRadixPlain = -1;
cudaError_t fftlen_create(FFTLen &L, int len, int variant = 0);
void fftlen_destroy(FFTLen &L);

template <typename T>
cudaError_t launch_rows_r2c(const T *in, long inPitch, long inBatch, int inCols, int nRows, void *out,
                            long outPitch, long outBatch, const FFTLen &Lx, int nBatch, cudaStream_t st);
template <typename T>
cudaError_t launch_cols(void *spec, long pitch, long batch, int nColsC, int nRowsIn, int nRowsOut,
                        const void *H, long hPitch, const FFTLen &Ly, T scale, int mode, int nBatch,
                        cudaStream_t st, int cpbOverride = 0, long hBatch = 0, int hDiv = 1,
                        const int *hMap = nullptr, int threadsOverride = 0);
// Column pass of the FP32 convolution (k_cols32.cu): mode 1 multiplies by H,
// mode 2 by conj(H); pitch and hPitch even (16-byte rows pieces); cpb
// columns per CTA in {1, 2, 4, 8} (0: automatic), threads 0: automatic.
cudaError_t launch_cols32(void *spec, long pitch, long batch, int nColsC, int nRowsIn, int nRowsOut, const void *H,
                          long hPitch, const FFTLen &Ly, float scale, int mode, int nBatch, cudaStream_t st,
                          int cpb = 0, long hBatch = 0, int hDiv = 1, const int *hMap = nullptr, int threads = 0);
size_t cols32_smem(int Ly, int cpb);
size_t cols32_fused_smem(int Ly, int cpb);
void cols32_prepare_kernels();
// complex pitch of a half spectrum of real length L: L/2 + 1 rounded up to
// even, so every row starts on a 16-byte boundary
inline int even_pitch(int L) { return ((L / 2 + 1) + 1) & ~1; }

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
  // subsampled pixels, computed beforehand by one warp each: sub[c][S*S] over
  // a box of S = 2 subHalf pixels around component c's centre (null: each
  // pixel's thread sums its subsamples itself)
  double *sub;
  int subHalf;
};

// Scratch size (doubles) of the subsampled-pixel table of nComp components on g.
size_t sub_table_size(const Grid64 &g, int nComp);

// 3-D (line-of-sight) components of a model: their indices in the component
// list; component c's CompF64::pad0 holds its position k3 in this list.
struct LosList64 {
  int n;
  int comp[kMaxComponents];
};
// los[k3 * (nCols*nRows) + pixel]: value of the k3-th 3-D component (FP64 QAGS per pixel)
cudaError_t launch_los64(const CompF64 *comps, const LosList64 &list, double *los, Grid64 g, int *flag,
                         cudaStream_t st);
// sum of one component's values over an xSize x ySize grid (FindTotalFluxes);
// nBlocks FP64 partials
cudaError_t launch_flux64(const CompF64 &c, int xSize, int ySize, double *partials, int nBlocks, int *flag,
                          cudaStream_t st);
// model pixels; 3-D components are read from 'los' (may be null without them)
cudaError_t launch_eval64(const CompF64 *comps, int nComp, double *model, long pitch, Grid64 g,
                          const double *los, cudaStream_t st);
// point sources the fast path evaluates (per model)
constexpr int kMaxPsFast = 8;

// per-component PointSource::oversamplingScale of one point-source pass
struct PsScales {
  int s[kMaxComponents];
};
// point sources after the convolution
cudaError_t launch_point_sources64(const CompF64 *comps, int nComp, double *model, long pitch, Grid64 g,
                                   PsfInterp<double> ip, const PsScales &scales, cudaStream_t st);
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
  long countStride;      // batched bootstrap: stride between the samples' counts (0: one sample)
  long dataStride;       // image stacks: data/weight stride between batch entries (0: one image)
  const int *entry;      // image stacks: image of batch entry b is entry[b] (null: b)
  int kind;              // 0 chi^2, 1 Cash
  int modelErrors;
  float effGain, sky, rnTerm;
  float psfSum, psfSumOs;
  // spectra and scratch
  void *spec;            // main half spectrum [B][Ly][specPitch] complex float
  void *rspec;           // region half spectrum
  // per-CTA partial sums, double-float (hi, lo) pairs: each thread sums its
  // few pixels in FP32 and the warp's 32 thread sums in FP32; every level
  // above (across warps, across CTAs) adds in double-float; the final value
  // is returned in FP64.
  // Layouts [B][quantity][partStride].
  float2 *statPart;      // quantities: S, sum of g * sum(PSF)
  float2 *gradPart;      // quantities: the nParams gradient entries
  int partStride;        // >= number of CTAs of any launch shape
  int nStatBlocks, nGradBlocks, nRegGradBlocks;
  double *stat;          // [B]
  double *grad;          // [B][nParams]
  // [B] completion counters: the last CTA of the final pass of an evaluation
  // (statistic pass without a gradient, else the gradient passes) adds the
  // partials up; zeroed by the first kernel of each evaluation
  unsigned *done;
  float *modelOut;       // optional: [B][N] model image (FP32) for inspection
  // subsampled pixels, precomputed warp-per-pixel over the whole GPU: for each
  // (batch, component, window) a square box of window pixels around the
  // component centre holds [value, 7 derivatives] averaged over the pixel's
  // subsamples (only pixels that subsample are written or read)
  float *subTab;         // [B][nComp][2 windows][boxArea(w)][8]
  int *subBox;           // [B][nComp][2][2]  box origin (col, row) in window coordinates
  int boxMain, boxReg;   // box sides (pixels)
  // oversampled region: the shared subsample lattice (null when the region's
  // scale does not divide its subsample count), [B][nComp][8][latSide^2],
  // over the box pixels within latHalf of the box centre
  float *lat;
  int latSide, latHalf;
  // 3-D (line-of-sight) components, when the model has any: per window
  // pixel the summed line-of-sight values and the adjoint r~, main window and
  // region window, [B][rows][cols] each (all null otherwise)
  float *losVal, *losRt, *rLosVal, *rLosRt;
  // their line-of-sight partitions kept from the forward pass for the gradient
  // pass ([B][nLos][window pixels][32] (lo, hi) pairs and counts), or null
  float *losPan, *rLosPan;
  int *losCnt, *rLosCnt;
  int nLos;
  // point sources, added after the convolution: component indices, the
  // interpolators of the main PSF and of the region's oversampled PSF, and
  // the gradient partials of the statistic CTAs, [B][nPs][4][partStride]
  // (d/dX0, d/dY0, d/dI_tot, d/dPA)
  int nPs;
  int psComp[kMaxPsFast];
  PsfInterp<float> psMain, psReg;
  float2 *psPart;
};

// CTAs per parameter vector of each line-of-sight kernel (grid-stride, one
// warp per pixel); the gradient kernel writes one partial per CTA.
constexpr int kLosCtas = 608;

// Optional per-stage CUDA events: an event is recorded on the launch stream
// after every kernel of the fast path (recorded into the graph when captured).
struct StageTimer {
  static constexpr int kMax = 48;
  cudaEvent_t ev[kMax];
  const char *names[kMax];
  int n = 0;
  // when set, only this stage is bracketed (ev[0] before it, ev[1] after), so
  // the timed graph carries two event nodes instead of one per kernel
  const char *only = nullptr;
};

// Launch shape of the fast-path kernels (chosen by the autotuner).
struct FastTune {
  int rowRpb = 3;        // window rows per CTA (eval, statistic, gradient kernels)
  int rowThreads = 256;  // threads per row CTA
  int colCpb = 0;        // half-spectrum columns per CTA (0: automatic)
  int colThreads = 0;    // threads per column CTA (0: one per complex point pair, <= 1024)
};

struct FastPlan {
  FastTune tune;
  StageTimer *timer = nullptr;
  // second stream for the oversampled-region pipeline (null: run serially),
  // the event that forks it from the main stream after the set-up, and those
  // that join it back at the end (statistic only / with the gradient)
  cudaStream_t side = nullptr;
  cudaEvent_t fork0 = nullptr, join0 = nullptr, join1 = nullptr;
  FastGeom g;
  const FFTLen *Lx, *Ly, *Rx, *Ry;  // main and region lengths
  const void *H, *Hr;               // FP32 PSF spectra (main, region)
  long hPitch, hrPitch;
  long hBatch = 0;                  // image stacks: spectrum stride between entries (0: one PSF)
  const int *hMap = nullptr;        // image stacks: PSF spectrum of batch entry b is hMap[b] (null: b)
};

// Forward-mode JtWJ buffers.  Parameters with slot[j] >= 0 get a derivative
// image; background parameters (slot -1) have dM/dtheta = sum(PSF).
struct JtwjArgs {
  void *dspec;       // [B*nD] main derivative spectra (complex float, specBatch each)
  void *drspec;      // [B*nD] region derivative spectra (rSpecBatch each)
  float *regDeriv;   // [B*nD][rRows][rCols] downsampled region derivatives
  const int *slot;   // [nParams]
  int nD;
  float2 *part;      // [B][Q][partStride] per-row partials (hi, lo), Q = nP(nP+1)/2 + nP + 1
  double *alpha;     // [B][nP][nP]  J^T J
  double *beta;      // [B][nP]      J^T dev
  double *stat;      // [B]          sum dev^2 (the fit statistic)
  float *jac;        // optional [B][nP + 1][nData]: d dev / d params, then the deviates
};

cudaError_t fast_jtwj(const FastPlan &p, const FastArgs &a, const JtwjArgs &J, int nBatch, cudaStream_t st);

// ------------------------------------------------------- ragged cutout sets
// Many cutouts of different sizes fitted with one model in one handle: each
// cutout keeps its own size, PSF and FFT plan (no padding to a common size),
// and every stage of an evaluation is ONE launch over all active cutouts --
// a flat grid whose CTA t serves the slot k with start[k] <= t < start[k+1]
// (binary search over the prefix sums of the slots' work counts).
// spectrum columns per CTA of a cutout set's column pass
constexpr int kRagColsPerCta = 4;

struct RagEntry {
  int nDataCols, nDataRows;  // the cutout
  int winCols, winRows;      // window W = N + P - 1
  int xOrig, yOrig;          // IRAF coordinate of window pixel (0,0)
  int Lx, Ly;                // padded FFT lengths (7-smooth, even)
  int pitch;                 // complex pitch of its half spectrum (even)
  int colGroups;             // column groups of its column pass
  long specOff;              // complex offset of its spectrum (specSize values)
  long specSize;             // Ly * pitch
  long dataOff;              // offset of its data / weight / model pixels
  long hOff;                 // complex offset of its PSF spectrum
  long rowOff;               // offset of its data rows in the per-row partials
  FFTPlan<float> rowPlan;    // Lx/2-point complex transform (rows)
  FFTPlan<float> colPlan;    // Ly-point transform (columns)
  FFTPlan<float> colPlanI;   // the same radices reversed (the column pass's inverse half; tw null: unfused)
  const cplx<float> *twL;    // Lx split twiddles
};

struct RagArgs {
  const RagEntry *ent;     // [entries]
  const int *act;          // [K] entry of slot k
  const int *start;        // [K + 1] prefix sums of the launch's work count per slot
  int K;
  int lines;               // column pass: spectra per entry (1, or nD derivative spectra)
  cplx<float> *spec;       // spectra (forward: specOff; derivatives: nD * specOff + j * specSize)
  const cplx<float> *H;    // PSF spectra (hOff)
  float *model;            // FP32 model images (dataOff)
  float2 *part;            // per-row partials (hi, lo) [Q][totalRows] (rowOff)
  long totalRows;
};

// slot of CTA t: the largest k with start[k] <= t (start[0] = 0)
__device__ __forceinline__ int rag_slot(const int *start, int K, int t) {
  int lo = 0, hi = K - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// work counts per slot of each ragged stage
enum RagWork { kRagWinRows = 0, kRagDataRows = 1, kRagCols = 2, kRagDerivCols = 3, kRagWorkKinds = 4 };

cudaError_t rag_jtwj(const FastArgs &a, RagArgs r, cplx<float> *dspec, const int *const starts[kRagWorkKinds],
                     const int totals[kRagWorkKinds], const int *slot, int nD, int maxM, int maxLy, int maxCols,
                     double *alpha, double *beta, double *stat, cudaStream_t st);
// shared memory of the ragged derivative and row-product kernels
size_t rag_jtwj_smem(int maxM, int nD, int nP, int maxCols);
cudaError_t launch_rag_cols(const RagArgs &r, int total, int maxLy, cudaStream_t st);
size_t fast_jtwj_smem(const FastPlan &p, int nD, int nP);
cudaError_t fast_forward(const FastPlan &p, const FastArgs &a, int nBatch, bool wantGrad, cudaStream_t st);
// one-time kernel attribute set-up (call before any stream capture)
void fast_prepare_kernels();
void fft_prepare_kernels();
int fast_stat_blocks(const FastGeom &g, const FastTune &t);
int fast_grad_blocks(const FastGeom &g, const FastTune &t);
int fast_reg_grad_blocks(const FastGeom &g, const FastTune &t);

}  // namespace imfit
