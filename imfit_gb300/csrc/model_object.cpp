// model_object.cpp -- host facade of the GB300 library: a C++ restatement of
// the reference's ModelObject state machine (core/model_object.cpp) whose
// compute calls go to the kernels in k_plain.cu / k_fft.cu / k_fast.cu, and
// the C ABI declared in include/imfit_gb300.h.
//
// Weight / mask / extra-term preparation stays on the host in FP64 with the
// reference's expressions (bit-identical by construction); the results are
// uploaded once at FinalSetupForFitting.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/imfit_gb300.h"
#include "kernels.h"
#include "lm.h"

namespace imfit {
cudaError_t launch_update_weights64(const double *model, const double *mask, double *weight, long nData,
                                    int nDataCols, int modelCols, int offR, int offC, double effGain, double sky,
                                    double rnTerm, cudaStream_t st);
cudaError_t launch_f64_to_f32(const double *in, float *out, long n, cudaStream_t st);
}  // namespace imfit

using namespace imfit;

namespace {

const char *kVersion = "imfit-gb300 0.1 (sm_103a)";

struct FuncInfo {
  std::string name;
  int type;
  int nParams;
  int subsample;
  int method = PSF_BICUBIC;  // point sources: the optional parameter "method"
  std::vector<std::string> paramNames;
};

bool lookup_function(const std::string &n, FuncInfo &f) {
  // core/add_functions.cpp:170-248 (config names) and each class's PARAM_LABELS
  static const std::map<std::string, std::pair<int, std::vector<std::string>>> reg = {
      {"Sersic", {F_SERSIC, {"PA", "ell", "n", "I_e", "r_e"}}},
      {"Exponential", {F_EXP, {"PA", "ell", "I_0", "h"}}},
      {"FlatSky", {F_FLATSKY, {"I_sky"}}},
      {"GaussianRing", {F_GRING, {"PA", "ell", "A", "R_ring", "sigma_r"}}},
      {"Moffat", {F_MOFFAT, {"PA", "ell", "I_0", "fwhm", "beta"}}},
      {"Gaussian", {F_GAUSS, {"PA", "ell", "I_0", "sigma"}}},
      {"ExponentialDisk3D", {F_EXPDISK3D, {"PA", "inc", "J_0", "h", "n", "z_0"}}},
      {"FerrersBar3D", {F_FERRERS3D, {"PA", "inc", "barPA", "J_0", "R_bar", "q", "q_z", "n"}}},
      {"PointSource", {F_POINTSOURCE, {"I_tot"}}},
      {"PointSourceRot", {F_POINTSOURCEROT, {"PA", "I_tot"}}},
      {"TiltedSkyPlane", {F_TILTEDSKY, {"I_0", "m_x", "m_y"}}},
  };
  auto it = reg.find(n);
  if (it == reg.end()) return false;
  f.name = n;
  f.type = it->second.first;
  f.paramNames = it->second.second;
  f.nParams = (int)f.paramNames.size();
  f.subsample = (f.type == F_EXPDISK3D || f.type == F_FERRERS3D || is_point_source(f.type)) ? 0 : 1;
  return true;
}

// Derivative at every knot of the natural cubic spline through v[k*stride],
// k < n, unit knot spacing (second derivatives M from the tridiagonal system
// M_{k-1} + 4 M_k + M_{k+1} = 6 (v_{k+1} - 2 v_k + v_{k-1}), M_0 = M_{n-1} = 0).
void spline_knot_derivs(const double *v, long stride, int n, double *out) {
  std::vector<double> M(n, 0.0), c(n, 0.0), d(n, 0.0);
  if (n > 2) {
    const int m = n - 2;
    for (int i = 0; i < m; i++) {
      const int k = i + 1;
      double rhs = 6.0 * (v[(k + 1) * stride] - 2.0 * v[k * stride] + v[(k - 1) * stride]);
      double diag = 4.0;
      if (i > 0) {
        const double w = 1.0 / c[i - 1];
        diag -= w;
        rhs -= w * d[i - 1];
      }
      c[i] = diag;
      d[i] = rhs;
    }
    M[m] = d[m - 1] / c[m - 1];
    for (int i = m - 2; i >= 0; i--) M[i + 1] = (d[i] - M[i + 2]) / c[i];
  }
  for (int k = 0; k < n - 1; k++)
    out[k * stride] = (v[(k + 1) * stride] - v[k * stride]) - (2.0 * M[k] + M[k + 1]) / 6.0;
  out[(n - 1) * stride] = (v[(n - 1) * stride] - v[(n - 2) * stride]) + (M[n - 2] + 2.0 * M[n - 1]) / 6.0;
}

// Host tables of a PSF interpolator (psf_interp.cuh): bicubic -> z, z_x, z_y,
// z_xy (z_xy the x-spline derivative of z_y); Lanczos -> the PSF.
std::vector<double> psf_interp_tables(int kind, const double *psf, int nc, int nr) {
  const long np = (long)nc * nr;
  if (kind != PSF_BICUBIC) return std::vector<double>(psf, psf + np);
  std::vector<double> t(4 * np);
  double *z = t.data(), *zx = z + np, *zy = zx + np, *zxy = zy + np;
  std::copy(psf, psf + np, z);
  for (int r = 0; r < nr; r++) spline_knot_derivs(z + (long)r * nc, 1, nc, zx + (long)r * nc);
  for (int c = 0; c < nc; c++) spline_knot_derivs(z + c, nc, nr, zy + c);
  for (int r = 0; r < nr; r++) spline_knot_derivs(zy + (long)r * nc, 1, nc, zxy + (long)r * nc);
  return t;
}

// Kahan-summed normalisation (core/convolver.cpp:296-311, core/model_object.cpp:2581-2594)
double kahan_sum(const double *v, long n) {
  double s = 0.0, err = 0.0, adj, tmp;
  for (long k = 0; k < n; k++) {
    adj = v[k] - err;
    tmp = s + adj;
    err = (tmp - s) - adj;
    s = tmp;
  }
  return s;
}

// MT19937 (Matsumoto & Nishimura 1998) as used by the reference's bootstrap
// (core/mersenne_twister.cpp:60-166).
struct MT19937 {
  unsigned long mt[624];
  int mti = 625;
  void seed(unsigned long s) {
    mt[0] = s & 0xffffffffUL;
    for (int i = 1; i < 624; i++) mt[i] = (1812433253UL * (mt[i - 1] ^ (mt[i - 1] >> 30)) + i) & 0xffffffffUL;
    mti = 624;
  }
  unsigned long next() {
    static const unsigned long mag01[2] = {0x0UL, 0x9908b0dfUL};
    unsigned long y;
    if (mti >= 624) {
      if (mti == 625) seed(5489UL);
      int kk;
      for (kk = 0; kk < 227; kk++) {
        y = (mt[kk] & 0x80000000UL) | (mt[kk + 1] & 0x7fffffffUL);
        mt[kk] = mt[kk + 397] ^ (y >> 1) ^ mag01[y & 1UL];
      }
      for (; kk < 623; kk++) {
        y = (mt[kk] & 0x80000000UL) | (mt[kk + 1] & 0x7fffffffUL);
        mt[kk] = mt[kk - 227] ^ (y >> 1) ^ mag01[y & 1UL];
      }
      y = (mt[623] & 0x80000000UL) | (mt[0] & 0x7fffffffUL);
      mt[623] = mt[396] ^ (y >> 1) ^ mag01[y & 1UL];
      mti = 0;
    }
    y = mt[mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680UL;
    y ^= (y << 15) & 0xefc60000UL;
    y ^= (y >> 18);
    return y & 0xffffffffUL;
  }
  double real2() { return (double)next() * (1.0 / 4294967296.0); }
};

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t reserve(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) n = count;
    return e;
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

struct Region {
  int x1, y1, nBaseCols, nBaseRows, scale;
  int nPsfCols, nPsfRows;
  std::vector<double> psf;  // normalised as the region's Convolver does
  std::vector<double> psfRaw;  // as given: the region's bicubic point-source interpolator reads it
  DevBuf<double> psTab;        // that interpolator's tables
  PsfInterp<double> ps64{};
  double psfSum = 1.0;
  int nModelCols, nModelRows;
  long nModelVals;
  FFTLen Lx, Ly;
  DevBuf<double> model;
  DevBuf<double> spec;   // complex, Ly x (Lx/2+1)
  DevBuf<double> H;      // complex
  int nColsSub, nRowsSub;
};

struct Captured {
  int nBatch = -1;
  const void *p = nullptr, *s = nullptr, *g = nullptr;
  cudaGraphExec_t exec = nullptr;
};

}  // namespace

struct imfit_model_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string lastError;

  // functions
  std::vector<FuncInfo> funcs;
  std::vector<int> setStart;
  bool setsDefined = false;
  int nParamsTot = 0;
  std::vector<int> paramOffset, x0Index;
  std::vector<std::string> paramNames;

  // PSF / model grid
  bool doConv = false;
  int nPsfCols = 0, nPsfRows = 0;
  std::vector<double> psf;  // normalised (Convolver) copy
  // point sources: per function PointSource::oversamplingScale (1 until an
  // oversampled region has been computed, then that region's scale -- the
  // reference never resets it, core/model_object.cpp:1190-1192), and the
  // ModelObject's interpolator of the (normalised) PSF, of the first point
  // source's kind (core/model_object.cpp:294-305, 345-381)
  std::vector<int> psScale;
  int nPointSources = 0;
  DevBuf<double> dPsTab;
  PsfInterp<double> ps64{};
  int psKind = 0;
  // fast path: FP32 interpolator tables, the component descriptors as on the
  // device (their psScale follows psScale), the gradient partials
  DevBuf<float> dPsTab32, dPsRegTab32;
  DevBuf<float2> dPsPart;
  PsfInterp<float> psMain32{}, psReg32{};
  std::vector<CompDesc> hDesc;
  bool psfNormalize = true;
  double psfSum = 1.0;
  bool modelSetupDone = false, modelComputed = false;
  int nDataCols = 0, nDataRows = 0, nModelCols = 0, nModelRows = 0;
  long nDataVals = 0, nValid = 0, nModelVals = 0;

  // data & statistic state (host, FP64, reference semantics)
  std::vector<double> data, weight, mask, extra;
  bool dataValsSet = false, weightValsSet = false, maskExists = false;
  bool dataErrors = true, modelErrors = false, externalErrors = false;
  bool useCash = false, pmlr = false, doBootstrap = false, finalSetupDone = false;
  double gain = 1.0, readNoise = 0.0, expTime = 1.0, sky = 0.0, effGain = 1.0, rnAduSq = 0.0;
  int nCombined = 1;
  std::vector<long> bootIdx;
  MT19937 rng;

  std::vector<Region *> regions;

  // plain FP64 device state
  FFTLen Lx, Ly;
  DevBuf<double> dModel, dSpec, dH, dData, dWeight, dMask, dExtra, dDev, dDev2, dPart, dRes;
  DevBuf<long> dBoot;
  DevBuf<CompF64> dComps;
  std::vector<CompF64> hComps;
  // 3-D (line-of-sight) components: per-pixel values computed before the pixel sum
  LosList64 losList{};
  DevBuf<double> dLos;
  DevBuf<double> dSub;  // subsampled-pixel table of the plain path (k_sub64)
  DevBuf<int> dLosFlag;
  int *hLosFlag = nullptr;  // pinned copy of the "list too short" flag
  double *hPinned = nullptr;  // pinned scratch for small transfers
  size_t hPinnedN = 0;
  // host-buffer fast evaluations: parameters in, statistics and gradients out
  // through mapped page-locked memory the kernels read and write directly
  // (no copy operations around the evaluation)
  double *hMapped = nullptr, *dMapped = nullptr;
  size_t hMappedN = 0;

  // fast FP32 device state
  bool fastReady = false;
  FastGeom fg{};
  FFTLen Fx, Fy, FRx, FRy;
  DevBuf<float> dH32, dHr32, dData32, dW32, dExtra32, dCount32, dBg, dModelOut;
  DevBuf<float> dCountBatch;  // batched bootstrap: [sample][data pixel] multiplicities
  int bootBatch = 0;          // number of samples while a batched bootstrap fit runs
  DevBuf<float> dSpec32, dRSpec32;  // complex
  DevBuf<CompDesc> dDesc;
  DevBuf<CompF32> dComps32;
  DevBuf<float> dSubTab;
  DevBuf<int> dSubBox;
  DevBuf<float> dLat;  // oversampled region's subsample lattice
  DevBuf<double> dParams, dStat, dGrad;
  DevBuf<float2> dStatPart, dGradPart;
  // image stack (fast path only): batch entry b has its own image, weights and PSF
  struct Stack {
    int n = 0, pc = 0, pr = 0;
    std::vector<float> data, weight;  // n x nDataVals
    std::vector<double> psf;          // n x pc*pr, normalised
  } stack;
  // image-stack subset being evaluated: image of batch entry b (device), or null
  DevBuf<int> dEntry;
  const int *curEntry = nullptr;
  // 3-D components: per window pixel line-of-sight values and adjoint r~
  bool hasLos = false;
  DevBuf<float> dLosVal32, dLosRt32, dRLosVal32, dRLosRt32;
  // kept line-of-sight partitions (null when they would exceed kLosKeepBytes)
  DevBuf<float> dLosPan, dRLosPan;
  DevBuf<int> dLosCnt, dRLosCnt;
  bool losKeep = false;
  static constexpr size_t kLosKeepBytes = 8ull << 30;
  int nLosComps() const {
    int k = 0;
    for (auto &f : funcs) k += (f.type == F_EXPDISK3D || f.type == F_FERRERS3D);
    return k;
  }
  // forward-mode JtWJ state: derivative slot per parameter (-1: background)
  // ragged cutout set (imfit_SetupCutouts): every cutout its own size, PSF and
  // FFT plan; evaluations are one launch per stage over the active cutouts
  struct RagSet {
    int n = 0;
    std::vector<RagEntry> ent;
    std::map<int, std::unique_ptr<FFTLen>> lens;
    long totalPix = 0, totalSpec = 0, totalRows = 0, totalH = 0;
    int maxM = 0, maxLy = 0, maxCols = 0;
    std::vector<int> work;  // act, then the prefix arrays, uploaded per evaluation
    ~RagSet() {
      for (auto &kv : lens) fftlen_destroy(*kv.second);
    }
  } rag;
  DevBuf<RagEntry> dRagEnt;
  DevBuf<float> dRagData, dRagW, dRagH, dRagModel, dRagPart, dRagSpec, dRagDSpec, dRagBg, dRagSubTab;
  DevBuf<CompF32> dRagComps;
  DevBuf<int> dRagSubBox, dRagWork, dRagSlot;
  DevBuf<double> dRagParams, dRagS, dRagA, dRagB;
  DevBuf<CompDesc> dRagDesc;
  int ragNDeriv = 0;
  std::vector<int> hRagSlot;
  std::vector<int> hSlot;
  int nDeriv = 0, jtwjCap = 0;
  DevBuf<int> dSlot;
  DevBuf<float> dDSpec32, dDRSpec32, dRegDeriv, dJPart;
  DevBuf<unsigned> dDone;
  DevBuf<double> dAlpha, dBeta;
  FastTune tune;
  std::map<int, FastTune> tuned;  // per batch size
  bool autotune = true;
  bool hasFixedTune = false;  // imfit_SetLaunchShape
  FastTune fixedTune;
  // FFT plan of the fast path: padded length = the fftCand-th smallest
  // 7-smooth even length >= the window (within 10 %), radix order fftVariant
  // (radix_schedule); chosen by the autotuner unless pinned (imfit_SetFFTPlan)
  int fftCand = 0, fftVariant = 0;
  bool fftPinned = false, fftTuned = false;
  int fftTunedB = 0;  // batch size the FFT plan was tuned at
  static constexpr int kFftCandidates = 3;
  int fftLength(int w) const {
    int c[kFftCandidates];
    const int n = smooth_candidates(w, true, kFftCandidates, 1.1, c);
    return c[std::min(fftCand, n - 1)];
  }
  int fastCap = 0;
  bool useGraphs = true;
  Captured graph;
  StageTimer timer;
  bool timing = false;
  std::string timingStage;           // empty: time every kernel (serially)
  cudaStream_t side = nullptr;       // oversampled-region pipeline
  cudaEvent_t forkEv[2] = {nullptr, nullptr}, joinEv[2] = {nullptr, nullptr};
  bool concurrent = true;

  ~imfit_model_s() {
    for (Region *r : regions) {
      fftlen_destroy(r->Lx);
      fftlen_destroy(r->Ly);
      delete r;
    }
    fftlen_destroy(Lx);
    fftlen_destroy(Ly);
    fftlen_destroy(Fx);
    fftlen_destroy(Fy);
    fftlen_destroy(FRx);
    fftlen_destroy(FRy);
    if (graph.exec) cudaGraphExecDestroy(graph.exec);
    if (timing)
      for (int i = 0; i < StageTimer::kMax; i++) cudaEventDestroy(timer.ev[i]);
    if (hPinned) cudaFreeHost(hPinned);
    if (hMapped) cudaFreeHost(hMapped);
    if (hLosFlag) cudaFreeHost(hLosFlag);
    for (int i = 0; i < 2; i++) {
      if (forkEv[i]) cudaEventDestroy(forkEv[i]);
      if (joinEv[i]) cudaEventDestroy(joinEv[i]);
    }
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
  }

  int fail(int code, const std::string &msg) {
    lastError = msg;
    return code;
  }
  int cuda_fail(cudaError_t e, const char *where) {
    lastError = std::string(where) + ": " + cudaGetErrorString(e);
    return (e == cudaErrorMemoryAllocation) ? IMFIT_E_NOMEM : IMFIT_E_CUDA;
  }
  double *pinned(size_t n) {
    if (n > hPinnedN) {
      if (hPinned) cudaFreeHost(hPinned);
      hPinned = nullptr;
      if (cudaMallocHost(&hPinned, sizeof(double) * n) != cudaSuccess) {
        hPinnedN = 0;
        return nullptr;
      }
      hPinnedN = n;
    }
    return hPinned;
  }

  long modelIndex(long z) const {
    if (!doConv) return z;
    long row = z / nDataCols, col = z - row * nDataCols;
    return (long)nModelCols * (nPsfRows + row) + nPsfCols + col;
  }

  // -------------------------------------------------------------- setup
  int defineSets(const int *starts, int n) {
    if (funcs.empty()) return fail(IMFIT_E_STATE, "DefineFunctionSets: no functions added");
    setStart.assign(funcs.size(), 0);
    setStart[0] = 1;
    for (int i = 0; i < n; i++) {
      if (starts[i] < 0 || starts[i] >= (int)funcs.size()) return fail(IMFIT_E_ARG, "bad function-set index");
      setStart[starts[i]] = 1;
    }
    paramOffset.assign(funcs.size(), 0);
    x0Index.assign(funcs.size(), 0);
    int off = 0, xi = 0;
    for (size_t f = 0; f < funcs.size(); f++) {
      if (setStart[f]) {
        xi = off;
        off += 2;
      }
      x0Index[f] = xi;
      paramOffset[f] = off;
      off += funcs[f].nParams;
    }
    nParamsTot = off;
    if (nParamsTot > kMaxParams) return fail(IMFIT_E_UNSUPPORTED, "too many parameters");
    setsDefined = true;
    fastReady = false;
    return 0;
  }

  void populateNames() {
    paramNames.clear();
    for (size_t f = 0; f < funcs.size(); f++) {
      if (setStart[f]) {
        paramNames.push_back("X0");
        paramNames.push_back("Y0");
      }
      for (auto &s : funcs[f].paramNames) paramNames.push_back(s);
    }
  }

  // FP64 spectrum of a real Ly x Lx array (host) via the device FFT kernels
  int spectrum64(const std::vector<double> &padded, const FFTLen &fx, const FFTLen &fy, DevBuf<double> &H) {
    const int nc = fx.L / 2 + 1;
    DevBuf<double> tmp;
    cudaError_t e = tmp.reserve(padded.size());
    if (!e) e = H.reserve(2 * (size_t)fy.L * nc);
    if (!e) e = cudaMemcpyAsync(tmp.p, padded.data(), sizeof(double) * padded.size(), cudaMemcpyHostToDevice, stream);
    if (!e) e = launch_rows_r2c<double>(tmp.p, fx.L, 0, fx.L, fy.L, H.p, nc, 0, fx, 1, stream);
    if (!e) e = launch_cols<double>(H.p, nc, 0, nc, fy.L, fy.L, nullptr, 0, fy, 1.0, 0, 1, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "PSF spectrum");
    return 0;
  }

  // padded PSF with the centre pixel (P/2) wrapped to (0,0): ShiftAndWrapPSF
  // (core/convolver.cpp:421-441)
  static std::vector<double> wrap_psf(const std::vector<double> &p, int pc, int pr, int Lx, int Ly) {
    std::vector<double> out((size_t)Lx * Ly, 0.0);
    const int cx = pc / 2, cy = pr / 2;
    for (int i = 0; i < pr; i++)
      for (int j = 0; j < pc; j++) {
        const int dc = (Lx - cx + j) % Lx, dr = (Ly - cy + i) % Ly;
        out[(size_t)dr * Lx + dc] = p[(size_t)i * pc + j];
      }
    return out;
  }

  int setupModelImage(int nc, int nr) {
    if (nc < 1 || nr < 1) return fail(IMFIT_E_ARG, "SetupModelImage: bad size");
    nDataCols = nc;
    nDataRows = nr;
    nDataVals = (long)nc * nr;
    if (doConv) {
      nModelCols = nc + 2 * nPsfCols;
      nModelRows = nr + 2 * nPsfRows;
      // reference padding N_model + P - 1 (core/convolver.cpp:217-219), rounded up to a 7-smooth size
      int e1 = fftlen_create(Lx, smooth_size(nModelCols + nPsfCols - 1, true), kRadixPlain);
      int e2 = fftlen_create(Ly, smooth_size(nModelRows + nPsfRows - 1, true), kRadixPlain);
      if (e1 || e2) return fail(IMFIT_E_CUDA, "FFT tables");
      int st = spectrum64(wrap_psf(psf, nPsfCols, nPsfRows, Lx.L, Ly.L), Lx, Ly, dH);
      if (st) return st;
      cudaError_t e = dSpec.reserve(2 * (size_t)Ly.L * (Lx.L / 2 + 1));
      if (e) return cuda_fail(e, "spectrum buffer");
    } else {
      nModelCols = nc;
      nModelRows = nr;
    }
    nModelVals = (long)nModelCols * nModelRows;
    cudaError_t e = dModel.reserve(nModelVals);
    if (e) return cuda_fail(e, "model buffer");
    modelSetupDone = true;
    fastReady = false;
    return 0;
  }

  int addRegion(const double *p, int pc, int pr, int scale, int x1, int x2, int y1, int y2, int normalize) {
    if (!modelSetupDone) return fail(IMFIT_E_STATE, "AddOversampledPsfInfo: SetupModelImage not called");
    if (pc < 1 || pr < 1 || scale < 1 || x1 >= x2 || y1 >= y2) return fail(IMFIT_E_ARG, "bad oversampled region");
    for (long i = 0; i < (long)pc * pr; i++)
      if (!std::isfinite(p[i])) return fail(IMFIT_E_ARG, "Oversampled PSF image has non-finite values");
    if (x1 < 1) x1 = 1;
    if (y1 < 1) y1 = 1;
    if (x2 > nDataCols) x2 = nDataCols;
    if (y2 > nDataRows) y2 = nDataRows;
    Region *r = new Region();
    r->x1 = x1;
    r->y1 = y1;
    r->nBaseCols = x2 - x1 + 1;
    r->nBaseRows = y2 - y1 + 1;
    r->scale = scale;
    r->nPsfCols = pc;
    r->nPsfRows = pr;
    r->psf.assign(p, p + (size_t)pc * pr);
    r->psfRaw = r->psf;
    if (normalize) {
      const double s = kahan_sum(r->psf.data(), (long)r->psf.size());
      for (auto &v : r->psf) v = v / s;
    }
    r->psfSum = 0.0;
    for (double v : r->psf) r->psfSum += v;
    r->nModelCols = r->nBaseCols * scale + 2 * pc;
    r->nModelRows = r->nBaseRows * scale + 2 * pr;
    r->nModelVals = (long)r->nModelCols * r->nModelRows;
    r->nColsSub = (r->nModelCols - 2 * pc) / scale;
    r->nRowsSub = (r->nModelCols - 2 * pr) / scale;  // core/downsample.cpp:79 uses the column count
    // the reference reads region-model rows up to (nRowsSub)*k + pr - 1 and
    // writes main pixels up to row y1-1+P+nRowsSub-1: both must stay in range
    const int lastRow = (r->nRowsSub - 1) * scale + pr + scale - 1;
    const int pcm = doConv ? nPsfCols : 0, prm = doConv ? nPsfRows : 0;
    if (r->nRowsSub < 1 || lastRow >= r->nModelRows || (y1 - 1 + prm + r->nRowsSub) > nModelRows ||
        (x1 - 1 + pcm + r->nColsSub) > nModelCols) {
      delete r;
      return fail(IMFIT_E_UNSUPPORTED,
                  "oversampled region shape would make DownsampleAndReplace read/write outside its images");
    }
    int e1 = fftlen_create(r->Lx, smooth_size(r->nModelCols + pc - 1, true), kRadixPlain);
    int e2 = fftlen_create(r->Ly, smooth_size(r->nModelRows + pr - 1, true), kRadixPlain);
    if (e1 || e2) {
      delete r;
      return fail(IMFIT_E_CUDA, "FFT tables");
    }
    int st = spectrum64(wrap_psf(r->psf, pc, pr, r->Lx.L, r->Ly.L), r->Lx, r->Ly, r->H);
    if (st) {
      delete r;
      return st;
    }
    cudaError_t e = r->model.reserve(r->nModelVals);
    if (!e) e = r->spec.reserve(2 * (size_t)r->Ly.L * (r->Lx.L / 2 + 1));
    if (e) {
      delete r;
      return cuda_fail(e, "region buffers");
    }
    regions.push_back(r);
    fastReady = false;
    return 0;
  }

  // GenerateErrorVector (core/model_object.cpp:642-673)
  void generateErrorVector() {
    weight.assign(nDataVals, 0.0);
    for (long z = 0; z < nDataVals; z++) {
      double tf = data[z] + sky;
      if (tf < 0.0) tf = 0.0;
      const double ns = tf / effGain + nCombined * rnAduSq;
      weight[z] = 1.0 / sqrt(ns);
    }
    weightValsSet = true;
  }

  // FinalSetupForFitting (core/model_object.cpp:967-1079)
  int finalSetup() {
    if (!dataValsSet) return fail(IMFIT_E_STATE, "FinalSetupForFitting: no image data");
    int ret = 0;
    const long n = nDataVals;
    if (!maskExists) {
      mask.assign(n, 1.0);
      maskExists = true;
    }
    for (long z = 0; z < n; z++)
      if (mask[z] > 0.0 && !std::isfinite(data[z])) {
        mask[z] = 0.0;
        nValid--;
      }
    if (!useCash && dataErrors && !externalErrors) generateErrorVector();
    if (useCash && pmlr) {
      // GenerateExtraCashTerms (core/model_object.cpp:695-709)
      for (long z = 0; z < n; z++) {
        const double dv = effGain * (data[z] + sky);
        extra[z] = (dv <= 0.0) ? 0.0 : dv * log(dv) - dv;
      }
    }
    if (externalErrors) {
      for (long z = 0; z < n; z++)
        if (mask[z] > 0.0 && !std::isfinite(weight[z])) {
          mask[z] = 0.0;
          weight[z] = 0.0;
          nValid--;
        }
    }
    // ApplyMask (core/model_object.cpp:794-816)
    if (weightValsSet && maskExists) {
      for (long z = 0; z < n; z++) {
        double nv = mask[z] * weight[z];
        if (!std::isfinite(nv) && mask[z] == 0.0) nv = 0.0;
        weight[z] = nv;
      }
    }
    // CheckWeightVector (core/model_object.cpp:2508-2550)
    bool nonfinite = false, negative = false;
    for (long z = 0; z < n; z++)
      if (mask[z] > 0.0) {
        if (!std::isfinite(weight[z])) nonfinite = true;
        else if (weight[z] < 0.0) negative = true;
      }
    if (nonfinite || negative) ret = -1;
    // VetDataVector (core/model_object.cpp:2496-2506)
    bool bad = false;
    for (long z = 0; z < n; z++)
      if (!std::isfinite(data[z])) {
        if (mask[z] > 0.0) bad = true;
        else data[z] = 0.0;
      }
    if (bad) ret = -2;
    if (nValid < 1) ret = -3;
    // upload
    cudaError_t e = dData.reserve(n);
    if (!e) e = dWeight.reserve(n);
    if (!e) e = dMask.reserve(n);
    if (!e) e = dExtra.reserve(n);
    if (!e) e = dDev.reserve(n);
    if (!e) e = dDev2.reserve(n);
    if (!e) e = dPart.reserve(kStatBlocks * 8);
    if (!e) e = dRes.reserve(kMaxParams + 8);
    if (!e) e = cudaMemcpy(dData.p, data.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(dWeight.p, weight.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(dMask.p, mask.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    if (!e && !extra.empty()) e = cudaMemcpy(dExtra.p, extra.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    if (!e && extra.empty()) e = cudaMemset(dExtra.p, 0, sizeof(double) * n);
    if (e) return cuda_fail(e, "FinalSetupForFitting upload");
    finalSetupDone = true;
    fastReady = false;
    if (ret == -1) lastError = "bad values detected in weight vector";
    if (ret == -2) lastError = "bad (non-masked) data values";
    if (ret == -3) lastError = "not enough valid data values available for fitting";
    return ret;
  }

  // -------------------------------------------------------- plain path
  int checkEval() {
    if (stack.n) return fail(IMFIT_E_UNSUPPORTED, "the plain FP64 path takes one image per ModelObject, not a stack");
    if (!setsDefined) return fail(IMFIT_E_STATE, "DefineFunctionSets not called");
    if (!modelSetupDone) return fail(IMFIT_E_STATE, "SetupModelImage not called");
    if (int st = ensurePointSourceInterp()) return st;
    return 0;
  }

  void setupComps(const double *params, CompF64 *out) {
    double x0 = 0.0, y0 = 0.0;
    int k3 = 0;
    for (size_t f = 0; f < funcs.size(); f++) {
      if (setStart[f]) {
        x0 = params[x0Index[f]];
        y0 = params[x0Index[f] + 1];
      }
      comp_setup64(out[f], funcs[f].type, funcs[f].subsample, params + paramOffset[f], x0, y0);
      if (funcs[f].type == F_EXPDISK3D || funcs[f].type == F_FERRERS3D) out[f].pad0 = k3++;
    }
  }

  // the 3-D components of the model, in component order
  void buildLosList() {
    losList.n = 0;
    for (size_t f = 0; f < funcs.size(); f++)
      if (funcs[f].type == F_EXPDISK3D || funcs[f].type == F_FERRERS3D) losList.comp[losList.n++] = (int)f;
  }

  // line-of-sight values of the 3-D components on one model grid, then the pixel sum
  cudaError_t evalGrid(const CompF64 *dC, double *model, long pitch, const Grid64 &g) {
    return evalGridN(dC, (int)funcs.size(), losList, model, pitch, g);
  }
  cudaError_t evalGridN(const CompF64 *dC, int nC, const LosList64 &ll, double *model, long pitch,
                        const Grid64 &g0) {
    // subsampled pixels: a table filled one warp per pixel (scratch reused by
    // every grid; the launches are ordered on the one stream)
    Grid64 g = g0;
    g.subHalf = g.isRegion ? (int)std::ceil(10.0 / g.frac) + 1 : 11;
    cudaError_t e = dSub.reserve(std::max<size_t>(sub_table_size(g, nC), 1));
    if (e) return e;
    g.sub = dSub.p;
    if (ll.n == 0) return launch_eval64(dC, nC, model, pitch, g, nullptr, stream);
    const size_t need = (size_t)ll.n * g.nCols * g.nRows;
    e = dLos.reserve(need);
    if (!e) e = launch_los64(dC, ll, dLos.p, g, dLosFlag.p, stream);
    if (!e) e = launch_eval64(dC, nC, model, pitch, g, dLos.p, stream);
    return e;
  }

  // GetSingleFunctionImage (core/model_object.cpp:1241-1336): one function on
  // the model grid, convolved (and its oversampled regions computed with that
  // function alone), cropped to the data size.  Like the reference it leaves
  // that image in the model buffer.
  int singleFunctionImage(const double *params, int fi, double *out) {
    int st = checkEval();
    if (st) return st;
    const int nC = (int)funcs.size();
    if (fi < 0 || fi >= nC) return fail(IMFIT_E_ARG, "function index out of range");
    for (int j = 0; j < nParamsTot; j++)
      if (!std::isfinite(params[j])) return fail(IMFIT_E_ARG, "non-finite values in parameter vector");
    hComps.resize(nC);
    setupComps(params, hComps.data());
    CompF64 one = hComps[fi];
    LosList64 ll{};
    if (one.type == F_EXPDISK3D || one.type == F_FERRERS3D) {
      one.pad0 = 0;
      ll.n = 1;
      ll.comp[0] = 0;
    }
    cudaError_t e = dComps.reserve(std::max(nC, 1));
    if (!e && ll.n && !hLosFlag) e = cudaMallocHost(&hLosFlag, sizeof(int));
    if (!e && ll.n) e = dLosFlag.reserve(1);
    if (!e && ll.n) e = cudaMemsetAsync(dLosFlag.p, 0, sizeof(int), stream);
    if (!e) e = cudaMemcpyAsync(dComps.p, &one, sizeof(CompF64), cudaMemcpyHostToDevice, stream);
    Grid64 g{};
    g.nCols = nModelCols;
    g.nRows = nModelRows;
    g.pc = doConv ? nPsfCols : 0;
    g.pr = doConv ? nPsfRows : 0;
    const bool ps = is_point_source(one.type);
    if (!e) e = evalGridN(dComps.p, 1, ll, dModel.p, nModelCols, g);
    if (!e && doConv && !ps) e = conv64(dModel.p, nModelCols, nModelRows, Lx, Ly, dH.p, dSpec.p);
    if (!e && ps) e = launch_point_sources64(dComps.p, 1, dModel.p, nModelCols, g, ps64, mainScales(&fi, 1), stream);
    for (Region *r : regions) {
      if (e) break;
      Grid64 rg{};
      rg.nCols = r->nModelCols;
      rg.nRows = r->nModelRows;
      rg.pc = r->nPsfCols;
      rg.pr = r->nPsfRows;
      rg.isRegion = 1;
      rg.x1 = r->x1;
      rg.y1 = r->y1;
      rg.frac = 1.0 / r->scale;
      rg.off = 0.5 * rg.frac - 0.5;
      e = evalGridN(dComps.p, 1, ll, r->model.p, r->nModelCols, rg);
      if (!e) e = conv64(r->model.p, r->nModelCols, r->nModelRows, r->Lx, r->Ly, r->H.p, r->spec.p);
      if (!e && ps) {
        PsScales sc{};
        sc.s[0] = r->scale;
        e = launch_point_sources64(dComps.p, 1, r->model.p, r->nModelCols, rg, r->ps64, sc, stream);
        psScale[fi] = r->scale;
      }
      if (!e)
        e = launch_downsample64(r->model.p, r->nModelCols, r->nModelRows, r->nPsfCols, r->nPsfRows, dModel.p,
                                nModelCols, nModelRows, doConv ? nPsfCols : 0, doConv ? nPsfRows : 0, r->x1, r->y1,
                                r->scale, stream);
    }
    DevBuf<double> tmp;
    if (!e) e = tmp.reserve(nDataVals);
    if (!e)
      e = launch_crop64(dModel.p, nModelCols, doConv ? nPsfRows : 0, doConv ? nPsfCols : 0, nDataCols, nDataRows,
                        tmp.p, stream);
    if (!e) e = cudaMemcpyAsync(out, tmp.p, sizeof(double) * nDataVals, cudaMemcpyDeviceToHost, stream);
    if (!e && ll.n) e = cudaMemcpyAsync(hLosFlag, dLosFlag.p, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "GetSingleFunctionImage");
    if (ll.n) {
      st = losCheck();
      if (st) return st;
    }
    modelComputed = true;
    return 0;
  }

  // FindTotalFluxes (core/model_object.cpp:2415-2470): every function centred
  // on an xSize x ySize image; the analytic TotalFlux where the class has one
  // (Sersic func_sersic.cpp:246-251, Exponential func_exp.cpp:210-213,
  // Gaussian func_gaussian.cpp:216-219), otherwise the sum of its values over
  // that image (on the GPU, FP64); backgrounds count zero.
  int findTotalFluxes(const double *params, int xSize, int ySize, double *indiv, double *total) {
    constexpr double kPi = 3.14159265358979;  // the function classes' PI (func_sersic.cpp:65)
    if (!setsDefined) return fail(IMFIT_E_STATE, "DefineFunctionSets not called");
    if (xSize < 1 || ySize < 1) return fail(IMFIT_E_ARG, "bad image size");
    const int nC = (int)funcs.size();
    const double xc = 0.5 * xSize, yc = 0.5 * ySize;
    constexpr int kBlocks = 1024;
    DevBuf<double> part;
    cudaError_t e = part.reserve(kBlocks);
    if (!e) e = dLosFlag.reserve(1);
    if (!e && !hLosFlag) e = cudaMallocHost(&hLosFlag, sizeof(int));
    if (!e) e = cudaMemsetAsync(dLosFlag.p, 0, sizeof(int), stream);
    if (e) return cuda_fail(e, "FindTotalFluxes");
    std::vector<double> hp(kBlocks);
    double sum = 0.0;
    for (int f = 0; f < nC; f++) {
      const double *p = params + paramOffset[f];
      CompF64 c;
      comp_setup64(c, funcs[f].type, funcs[f].subsample, p, xc, yc);
      double flux = 0.0;
      const int t = funcs[f].type;
      if (t == F_FLATSKY || t == F_TILTEDSKY) {  // IsBackground: model_object.cpp:2449-2450
        flux = 0.0;
      } else if (t == F_SERSIC) {
        const double n = p[2], I_e = p[3], r_e = p[4], q = 1.0 - p[1], bn = sersic_bn(n);
        const double bn2n = pow(bn, 2.0 * n);
        const double L = 2 * kPi * n * exp(bn) * I_e * (r_e * r_e);
        flux = q * L * std::tgamma(2 * n) / bn2n;
      } else if (t == F_EXP) {
        flux = (1.0 - p[1]) * 2.0 * kPi * p[2] * p[3] * p[3];
      } else if (t == F_GAUSS) {
        flux = (1.0 - p[1]) * 2.0 * kPi * p[2] * p[3] * p[3];
      } else if (is_point_source(t)) {  // func_pointsource.cpp:241-244
        flux = (t == F_POINTSOURCE) ? p[0] : p[1];
      } else {
        e = launch_flux64(c, xSize, ySize, part.p, kBlocks, dLosFlag.p, stream);
        if (!e) e = cudaMemcpyAsync(hp.data(), part.p, sizeof(double) * kBlocks, cudaMemcpyDeviceToHost, stream);
        if (!e) e = cudaMemcpyAsync(hLosFlag, dLosFlag.p, sizeof(int), cudaMemcpyDeviceToHost, stream);
        if (!e) e = cudaStreamSynchronize(stream);
        if (e) return cuda_fail(e, "FindTotalFluxes");
        for (double v : hp) flux += v;
        if (*hLosFlag) {
          *hLosFlag = 0;
          return fail(IMFIT_E_UNSUPPORTED, "a line-of-sight integral needed more subintervals than the device "
                                           "QAGS list holds (64)");
        }
      }
      if (indiv) indiv[f] = flux;
      sum += flux;
    }
    if (total) *total = sum;
    return 0;
  }

  // after a synchronize: did a line-of-sight integral run out of subintervals?
  int losCheck() {
    if (losList.n && hLosFlag && *hLosFlag) {
      *hLosFlag = 0;
      cudaMemset(dLosFlag.p, 0, sizeof(int));
      return fail(IMFIT_E_UNSUPPORTED, "a line-of-sight integral needed more subintervals than the device "
                                       "QAGS list holds (64)");
    }
    return 0;
  }

  cudaError_t conv64(double *img, int nCols, int nRows, const FFTLen &fx, const FFTLen &fy, const double *H,
                     double *spec) {
    const int nc = fx.L / 2 + 1;
    cudaError_t e = launch_rows_r2c<double>(img, nCols, 0, nCols, nRows, spec, nc, 0, fx, 1, stream);
    if (!e) e = launch_cols<double>(spec, nc, 0, nc, nRows, nRows, H, nc, fy, 1.0 / ((double)fx.L * fy.L), 1, 1, stream);
    if (!e) e = launch_rows_c2r<double>(spec, nc, 0, nRows, img, nCols, 0, nCols, 1.0, fx, 1, stream);
    return e;
  }

  // Interpolator tables for the point sources (built on first use, again
  // after the PSF or a point source's method changes).
  int ensurePointSourceInterp() {
    if (!nPointSources) return 0;
    int kind = PSF_BICUBIC;
    for (auto &f : funcs)
      if (is_point_source(f.type)) {
        kind = f.method;
        break;
      }
    if (psKind != kind) {
      if (psf.empty()) return fail(IMFIT_E_STATE, "PointSource image function being used, but no PSF image was supplied");
      if (nPsfCols < 4 || nPsfRows < 4)
        return fail(IMFIT_E_ARG, "PSF image is too small for interpolation with PointSource functions (4 x 4 minimum)");
      std::vector<double> t = psf_interp_tables(kind, psf.data(), nPsfCols, nPsfRows);
      cudaError_t e = dPsTab.reserve(t.size());
      if (!e) e = cudaMemcpy(dPsTab.p, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice);
      if (e) return cuda_fail(e, "PSF interpolator");
      ps64 = PsfInterp<double>{kind, nPsfCols, nPsfRows, 0, (nPsfCols - 1) / 2.0, (nPsfRows - 1) / 2.0, dPsTab.p};
      psKind = kind;
    }
    for (Region *r : regions) {
      if (r->ps64.kind) continue;
      if (r->nPsfCols < 4 || r->nPsfRows < 4)
        return fail(IMFIT_E_ARG, "Oversampled PSF image is too small for interpolation with PointSource functions");
      std::vector<double> t = psf_interp_tables(PSF_BICUBIC, r->psfRaw.data(), r->nPsfCols, r->nPsfRows);
      cudaError_t e = r->psTab.reserve(t.size());
      if (!e) e = cudaMemcpy(r->psTab.p, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice);
      if (e) return cuda_fail(e, "oversampled PSF interpolator");
      r->ps64 = PsfInterp<double>{PSF_BICUBIC, r->nPsfCols, r->nPsfRows, 0, (r->nPsfCols - 1) / 2.0,
                                  (r->nPsfRows - 1) / 2.0, r->psTab.p};
    }
    return 0;
  }

  // point-source passes of components [c0, c0 + nC) of the device array dC,
  // whose function indices are fi[0..nC): main grid at each one's current
  // scale, then a region grid at the region's scale (the scale the components
  // keep afterwards)
  PsScales mainScales(const int *fi, int nC) {
    PsScales sc{};
    for (int c = 0; c < nC; c++) sc.s[c] = psScale[fi[c]];
    return sc;
  }

  // CreateModelImage (core/model_object.cpp:1103-1229) with comps already on the device
  cudaError_t enqueueModel(const CompF64 *dC) {
    buildLosList();
    cudaError_t e = cudaSuccess;
    if (losList.n && !hLosFlag) {
      // the flag accumulates over evaluations until losCheck() reads and clears it
      e = cudaMallocHost(&hLosFlag, sizeof(int));
      if (!e) e = dLosFlag.reserve(1);
      if (!e) e = cudaMemsetAsync(dLosFlag.p, 0, sizeof(int), stream);
      if (e) return e;
      *hLosFlag = 0;
    }
    Grid64 g{};
    g.nCols = nModelCols;
    g.nRows = nModelRows;
    g.pc = doConv ? nPsfCols : 0;
    g.pr = doConv ? nPsfRows : 0;
    e = evalGrid(dC, dModel.p, nModelCols, g);
    if (!e && doConv) e = conv64(dModel.p, nModelCols, nModelRows, Lx, Ly, dH.p, dSpec.p);
    const int nC = (int)funcs.size();
    std::vector<int> all(nC);
    for (int c = 0; c < nC; c++) all[c] = c;
    if (!e && nPointSources) e = launch_point_sources64(dC, nC, dModel.p, nModelCols, g, ps64, mainScales(all.data(), nC), stream);
    for (Region *r : regions) {
      if (e) break;
      Grid64 rg{};
      rg.nCols = r->nModelCols;
      rg.nRows = r->nModelRows;
      rg.pc = r->nPsfCols;
      rg.pr = r->nPsfRows;
      rg.isRegion = 1;
      rg.x1 = r->x1;
      rg.y1 = r->y1;
      rg.frac = 1.0 / r->scale;
      rg.off = 0.5 * rg.frac - 0.5;
      e = evalGrid(dC, r->model.p, r->nModelCols, rg);
      if (!e) e = conv64(r->model.p, r->nModelCols, r->nModelRows, r->Lx, r->Ly, r->H.p, r->spec.p);
      if (!e && nPointSources) {
        PsScales sc{};
        for (int c = 0; c < nC; c++) sc.s[c] = r->scale;
        e = launch_point_sources64(dC, nC, r->model.p, r->nModelCols, rg, r->ps64, sc, stream);
        for (int c = 0; c < nC; c++)
          if (is_point_source(funcs[c].type)) psScale[c] = r->scale;
      }
      if (!e)
        e = launch_downsample64(r->model.p, r->nModelCols, r->nModelRows, r->nPsfCols, r->nPsfRows, dModel.p,
                                nModelCols, nModelRows, doConv ? nPsfCols : 0, doConv ? nPsfRows : 0, r->x1, r->y1,
                                r->scale, stream);
    }
    if (!e && losList.n) e = cudaMemcpyAsync(hLosFlag, dLosFlag.p, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (!e && modelErrors && finalSetupDone)
      e = launch_update_weights64(dModel.p, dMask.p, dWeight.p, nDataVals, nDataCols, nModelCols,
                                  doConv ? nPsfRows : 0, doConv ? nPsfCols : 0, effGain, sky, nCombined * rnAduSq,
                                  stream);
    return e;
  }

  // finish = false: only enqueued (the caller synchronises and then calls
  // losCheck); a pageable source is staged by cudaMemcpyAsync before it
  // returns, so hComps may be reused at once
  int createModelImage(const double *params, bool finish = true) {
    int st = checkEval();
    if (st) return st;
    const int nC = (int)funcs.size();
    hComps.resize(nC);
    setupComps(params, hComps.data());
    cudaError_t e = dComps.reserve(nC);
    if (!e) e = cudaMemcpyAsync(dComps.p, hComps.data(), sizeof(CompF64) * nC, cudaMemcpyHostToDevice, stream);
    if (!e) e = enqueueModel(dComps.p);
    if (!e && finish) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "CreateModelImage");
    if (finish) {
      st = losCheck();
      if (st) return st;
    }
    modelComputed = true;
    return 0;
  }

  StatArgs64 statArgs(int kind) {
    StatArgs64 a{};
    a.model = dModel.p;
    a.data = dData.p;
    a.weight = dWeight.p;
    a.extra = dExtra.p;
    a.mask = dMask.p;
    a.boot = doBootstrap ? dBoot.p : nullptr;
    a.nz = doBootstrap ? nValid : nDataVals;
    a.nDataCols = nDataCols;
    a.modelCols = nModelCols;
    a.offR = doConv ? nPsfRows : 0;
    a.offC = doConv ? nPsfCols : 0;
    a.effGain = effGain;
    a.sky = sky;
    a.rnTerm = nCombined * rnAduSq;
    a.modelErrors = 0;  // weights are updated in place after each model
    a.kind = kind;
    return a;
  }

  int statKind() const { return useCash ? (pmlr ? 2 : 1) : 0; }

  int getFitStatistic(const double *params, double *out, int forceKind = -1) {
    if (!finalSetupDone) return fail(IMFIT_E_STATE, "FinalSetupForFitting not called");
    int st = createModelImage(params, false);
    if (st) return st;
    int kind = forceKind >= 0 ? forceKind : statKind();
    if (kind == 2) kind = 1;  // GetFitStatistic -> CashStatistic for PMLR (core/model_object.cpp:1620-1626)
    cudaError_t e = launch_statistic64(statArgs(kind), dPart.p, dRes.p, stream);
    double *h = pinned(8);
    if (!e) e = cudaMemcpyAsync(h, dRes.p, sizeof(double), cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "GetFitStatistic");
    st = losCheck();
    if (st) return st;
    *out = h[0];
    return 0;
  }

  int computeDeviates(double *y, const double *params) {
    if (!finalSetupDone) return fail(IMFIT_E_STATE, "FinalSetupForFitting not called");
    int st = createModelImage(params, false);
    if (st) return st;
    StatArgs64 a = statArgs(pmlr ? 2 : 0);
    cudaError_t e = launch_deviates64(a, dDev.p, nullptr, stream);
    if (!e) e = cudaMemcpyAsync(y, dDev.p, sizeof(double) * a.nz, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "ComputeDeviates");
    return losCheck();
  }

  // statistic + FD gradient (1 + nParams plain evaluations)
  int fdGradient(const double *params, double *stat, double *grad) {
    if (!finalSetupDone) return fail(IMFIT_E_STATE, "FinalSetupForFitting not called");
    int st = checkEval();
    if (st) return st;
    const int nP = nParamsTot, nC = (int)funcs.size();
    const double eps = sqrt(2.2204460e-16);  // MP_MACHEP0 (solvers/mpfit.h)
    std::vector<CompF64> all((size_t)(nP + 1) * nC);
    std::vector<double> x(params, params + nP), h(nP);
    setupComps(x.data(), all.data());
    for (int j = 0; j < nP; j++) {
      const double t = x[j];
      double hh = eps * fabs(t);
      if (hh == 0.0) hh = eps;
      h[j] = hh;
      x[j] = t + hh;
      setupComps(x.data(), all.data() + (size_t)(j + 1) * nC);
      x[j] = t;
    }
    cudaError_t e = dComps.reserve(all.size());
    if (!e) e = cudaMemcpyAsync(dComps.p, all.data(), sizeof(CompF64) * all.size(), cudaMemcpyHostToDevice, stream);
    const bool chi = !useCash;
    StatArgs64 a = statArgs(chi ? 0 : 1);
    if (!e) e = enqueueModel(dComps.p);
    if (!e) e = launch_statistic64(a, dPart.p, dRes.p, stream);
    if (chi && !e) e = launch_deviates64(statArgs(0), dDev.p, nullptr, stream);
    for (int j = 0; j < nP && !e; j++) {
      e = enqueueModel(dComps.p + (size_t)(j + 1) * nC);
      if (e) break;
      if (chi) {
        e = launch_deviates64(statArgs(0), dDev2.p, nullptr, stream);
        if (!e) e = launch_fd_dot64(dDev.p, dDev2.p, a.nz, 1.0 / h[j], dPart.p, dRes.p + 1 + j, stream);
      } else {
        e = launch_statistic64(a, dPart.p, dRes.p + 1 + j, stream);
      }
    }
    double *hb = pinned(nP + 1);
    if (!e) e = cudaMemcpyAsync(hb, dRes.p, sizeof(double) * (nP + 1), cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "FD gradient");
    st = losCheck();
    if (st) return st;
    *stat = hb[0];
    for (int j = 0; j < nP; j++) grad[j] = chi ? hb[1 + j] : (hb[1 + j] - hb[0]) / h[j];
    modelComputed = true;
    return 0;
  }

  // --------------------------------------------------------- fast path
  int prepareFast() {
    if (fastReady) return 0;
    if (!finalSetupDone) return fail(IMFIT_E_STATE, "FinalSetupForFitting not called");
    if (!setsDefined) return fail(IMFIT_E_STATE, "DefineFunctionSets not called");
    if (nPointSources > kMaxPsFast) return fail(IMFIT_E_UNSUPPORTED, "more than 8 point sources for the fast path");
    if (nPointSources && regions.size() > 1)
      return fail(IMFIT_E_UNSUPPORTED, "point sources with more than one oversampled region on the fast path");
    if (int st0 = ensurePointSourceInterp()) return st0;
    hasLos = false;
    for (auto &f : funcs)
      if (f.type == F_EXPDISK3D || f.type == F_FERRERS3D) hasLos = true;
    if (regions.size() > 1) return fail(IMFIT_E_UNSUPPORTED, "fast path supports at most one oversampled region");
    if ((int)funcs.size() > kMaxComponents) return fail(IMFIT_E_UNSUPPORTED, "too many components");
    if (stack.n && !regions.empty()) return fail(IMFIT_E_UNSUPPORTED, "image stacks do not take oversampled regions");
    const int pc = stack.n ? stack.pc : (doConv ? nPsfCols : 1), pr = stack.n ? stack.pr : (doConv ? nPsfRows : 1);
    std::vector<double> kp = stack.n ? std::vector<double>(stack.psf.begin(), stack.psf.begin() + (size_t)pc * pr)
                                     : (doConv ? psf : std::vector<double>{1.0});
    FastGeom &g = fg;
    g = FastGeom{};
    g.nDataCols = nDataCols;
    g.nDataRows = nDataRows;
    g.winCols = nDataCols + pc - 1;
    g.winRows = nDataRows + pr - 1;
    g.xOrig = 2 - pc + pc / 2;
    g.yOrig = 2 - pr + pr / 2;
    fftlen_destroy(Fx);
    fftlen_destroy(Fy);
    if (fftlen_create(Fx, fftLength(g.winCols), fftVariant) || fftlen_create(Fy, fftLength(g.winRows), fftVariant))
      return fail(IMFIT_E_CUDA, "FFT tables");
    if (Fx.L / 2 > 4096 || Fy.L > 4096) return fail(IMFIT_E_UNSUPPORTED, "image too large for the fast path");
    g.specPitch = even_pitch(Fx.L);
    g.specBatch = (long)Fy.L * g.specPitch;
    // PSF placed so that circular output (r,c) is the data pixel (r,c)
    int st = 0;
    if (stack.n) {
      const size_t hb = 2 * (size_t)Fy.L * even_pitch(Fx.L);
      cudaError_t e0 = dH32.reserve(hb * stack.n);
      if (e0) return cuda_fail(e0, "stack PSF spectra");
      for (int i = 0; i < stack.n && !st; i++)
        st = shiftedSpectrum32To(stack.psf.data() + (size_t)i * pc * pr, pc, pr, Fx, Fy, dH32.p + hb * i);
    } else {
      st = shiftedSpectrum32(kp, pc, pr, Fx, Fy, dH32);
    }
    if (st) return st;
    double ps = 0.0;
    for (double v : kp) ps += v;
    psfSumFast = ps;
    psfSumOsFast = 1.0;
    if (!regions.empty()) {
      Region *r = regions[0];
      const int k = r->scale;
      g.hasRegion = 1;
      g.rx0 = r->x1 - 1;
      g.ry0 = r->y1 - 1;
      g.rCols = r->nColsSub;
      g.rRows = r->nRowsSub;
      if (g.rRows > r->nBaseRows || g.rCols > r->nBaseCols || g.ry0 + g.rRows > nDataRows ||
          g.rx0 + g.rCols > nDataCols)
        return fail(IMFIT_E_UNSUPPORTED, "fast path needs the replaced region inside the region model and the image");
      g.rScale = k;
      g.rSubCols = g.rCols * k;
      g.rSubRows = g.rRows * k;
      g.rWinCols = g.rSubCols + r->nPsfCols - 1;
      g.rWinRows = g.rSubRows + r->nPsfRows - 1;
      g.rXBase = r->x1;
      g.rYBase = r->y1;
      g.rWinOffX = 1 + r->nPsfCols / 2 - r->nPsfCols;
      g.rWinOffY = 1 + r->nPsfRows / 2 - r->nPsfRows;
      const double frac = 1.0 / k;
      g.rFrac = (float)frac;
      g.rStartOff = (float)(0.5 * frac - 0.5);
      fftlen_destroy(FRx);
      fftlen_destroy(FRy);
      if (fftlen_create(FRx, fftLength(g.rWinCols), fftVariant) ||
          fftlen_create(FRy, fftLength(g.rWinRows), fftVariant))
        return fail(IMFIT_E_CUDA, "FFT tables");
      if (FRx.L / 2 > 4096 || FRy.L > 4096) return fail(IMFIT_E_UNSUPPORTED, "region too large for the fast path");
      g.rSpecPitch = even_pitch(FRx.L);
      g.rSpecBatch = (long)FRy.L * g.rSpecPitch;
      st = shiftedSpectrum32(r->psf, r->nPsfCols, r->nPsfRows, FRx, FRy, dHr32);
      if (st) return st;
      psfSumOsFast = r->psfSum;
    }
    // FP32 statistic inputs
    const long n = nDataVals;
    std::vector<float> f32(n);
    const size_t nAll = (size_t)n * (stack.n ? stack.n : 1);
    cudaError_t e = dData32.reserve(nAll);
    if (!e) e = dW32.reserve(nAll);
    if (!e) e = dExtra32.reserve(n);
    if (!e) e = dCount32.reserve(n);
    if (e) return cuda_fail(e, "fast buffers");
    if (stack.n) {
      e = cudaMemcpy(dData32.p, stack.data.data(), sizeof(float) * nAll, cudaMemcpyHostToDevice);
      if (!e) e = cudaMemcpy(dW32.p, stack.weight.data(), sizeof(float) * nAll, cudaMemcpyHostToDevice);
    } else {
      for (long z = 0; z < n; z++) f32[z] = (float)data[z];
      e = cudaMemcpy(dData32.p, f32.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
      for (long z = 0; z < n; z++) f32[z] = (float)weight[z];
      if (!e) e = cudaMemcpy(dW32.p, f32.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    }
    for (long z = 0; z < n; z++) f32[z] = extra.empty() ? 0.f : (float)extra[z];
    if (!e) e = cudaMemcpy(dExtra32.p, f32.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    if (!e) e = uploadCounts();
    // component descriptors
    std::vector<CompDesc> desc(funcs.size());
    for (size_t f = 0; f < funcs.size(); f++) {
      CompDesc &d = desc[f];
      d = CompDesc{};
      d.type = funcs[f].type;
      d.subsample = funcs[f].subsample;
      d.paramOffset = paramOffset[f];
      d.x0Index = x0Index[f];
      d.nParams = funcs[f].nParams;
      d.background = (funcs[f].type == F_FLATSKY) ? 1 : 0;
      d.psScale = psScale[f];
    }
    hDesc = desc;
    if (!e && nPointSources) {
      auto up = [&](const std::vector<double> &t64, DevBuf<float> &dst) {
        std::vector<float> t32(t64.begin(), t64.end());
        cudaError_t ee = dst.reserve(t32.size());
        if (!ee) ee = cudaMemcpy(dst.p, t32.data(), sizeof(float) * t32.size(), cudaMemcpyHostToDevice);
        return ee;
      };
      e = up(psf_interp_tables(psKind, psf.data(), nPsfCols, nPsfRows), dPsTab32);
      psMain32 = PsfInterp<float>{psKind, nPsfCols, nPsfRows, 0, (float)((nPsfCols - 1) / 2.0),
                                  (float)((nPsfRows - 1) / 2.0), dPsTab32.p};
      if (!e && !regions.empty()) {
        Region *r = regions[0];
        e = up(psf_interp_tables(PSF_BICUBIC, r->psfRaw.data(), r->nPsfCols, r->nPsfRows), dPsRegTab32);
        psReg32 = PsfInterp<float>{PSF_BICUBIC, r->nPsfCols, r->nPsfRows, 0, (float)((r->nPsfCols - 1) / 2.0),
                                   (float)((r->nPsfRows - 1) / 2.0), dPsRegTab32.p};
      }
    }
    if (!e) e = dDesc.reserve(desc.size());
    if (!e) e = cudaMemcpy(dDesc.p, desc.data(), sizeof(CompDesc) * desc.size(), cudaMemcpyHostToDevice);
    // derivative images for every parameter except constant backgrounds
    hSlot.assign(nParamsTot, 0);
    for (auto &d : desc)
      if (d.background) hSlot[d.paramOffset] = -1;
    nDeriv = 0;
    for (int j = 0; j < nParamsTot; j++)
      if (hSlot[j] >= 0) hSlot[j] = nDeriv++;
    if (!e) e = dSlot.reserve(std::max(nParamsTot, 1));
    if (!e) e = cudaMemcpy(dSlot.p, hSlot.data(), sizeof(int) * nParamsTot, cudaMemcpyHostToDevice);
    if (e) return cuda_fail(e, "fast setup upload");
    jtwjCap = 0;
    fastCap = 0;
    tuned.clear();
    if (graph.exec) {
      cudaGraphExecDestroy(graph.exec);
      graph = Captured{};
    }
    fastReady = true;
    return 0;
  }
  double psfSumFast = 1.0, psfSumOsFast = 1.0;

  cudaError_t uploadCounts() {
    if (!doBootstrap) return cudaSuccess;
    std::vector<float> cnt(nDataVals, 0.f);
    for (long i = 0; i < nValid; i++) cnt[bootIdx[i]] += 1.f;
    return cudaMemcpy(dCount32.p, cnt.data(), sizeof(float) * nDataVals, cudaMemcpyHostToDevice);
  }

  int shiftedSpectrum32(const std::vector<double> &p, int pc, int pr, const FFTLen &fx, const FFTLen &fy,
                        DevBuf<float> &H32) {
    cudaError_t e = H32.reserve(2 * (size_t)fy.L * even_pitch(fx.L));
    if (e) return cuda_fail(e, "FP32 PSF spectrum");
    return shiftedSpectrum32To(p.data(), pc, pr, fx, fy, H32.p);
  }

  // FP32 spectrum of one PSF (centre wrapped to (0,0)) written to dst, rows
  // at the even pitch even_pitch(fx.L) (the padding column zero)
  int shiftedSpectrum32To(const double *p, int pc, int pr, const FFTLen &fx, const FFTLen &fy, float *dst) {
    std::vector<double> pad((size_t)fx.L * fy.L, 0.0);
    for (int k = 0; k < pr; k++)
      for (int l = 0; l < pc; l++) {
        const int rr = ((k - pr + 1) % fy.L + fy.L) % fy.L;
        const int cc = ((l - pc + 1) % fx.L + fx.L) % fx.L;
        pad[(size_t)rr * fx.L + cc] = p[(size_t)k * pc + l];
      }
    DevBuf<double> H64;
    int st = spectrum64(pad, fx, fy, H64);
    if (st) return st;
    const size_t w = fx.L / 2 + 1, pitch = even_pitch(fx.L);
    const size_t nc = 2 * (size_t)fy.L * w;
    DevBuf<float> tmp;
    cudaError_t e = tmp.reserve(nc);
    if (!e) e = launch_f64_to_f32(H64.p, tmp.p, (long)nc, stream);
    if (!e) e = cudaMemsetAsync(dst, 0, sizeof(float) * 2 * pitch * fy.L, stream);
    if (!e)
      e = cudaMemcpy2DAsync(dst, sizeof(float) * 2 * pitch, tmp.p, sizeof(float) * 2 * w, sizeof(float) * 2 * w,
                            fy.L, cudaMemcpyDeviceToDevice, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "FP32 PSF spectrum");
    return 0;
  }

  int ensureFastCap(int B) {
    if (B <= fastCap) return 0;
    const FastGeom &g = fg;
    const int nP = nParamsTot, nC = (int)funcs.size();
    const int stride = partStride();
    cudaError_t e = dParams.reserve((size_t)B * nP);
    if (!e) e = dComps32.reserve((size_t)B * nC);
    if (!e) e = dBg.reserve((size_t)B * 2);
    if (!e) e = dSpec32.reserve(2 * (size_t)B * g.specBatch);
    if (!e && g.hasRegion) e = dRSpec32.reserve(2 * (size_t)B * g.rSpecBatch);
    if (!e) e = dStatPart.reserve((size_t)B * 2 * stride);
    if (!e) e = dGradPart.reserve((size_t)B * nP * stride);
    if (!e && nPointSources) e = dPsPart.reserve((size_t)B * 4 * nPointSources * stride);
    if (!e) e = dStat.reserve(B);
    if (!e) e = dDone.reserve(B);
    if (!e) e = cudaMemset(dDone.p, 0, sizeof(unsigned) * B);
    if (!e) e = dGrad.reserve((size_t)B * nP);
    const long area = (long)kBoxMain * kBoxMain + (long)boxReg() * boxReg();
    if (!e) e = dSubTab.reserve((size_t)B * nC * area * 8);
    if (!e) e = dSubBox.reserve((size_t)B * nC * 4);
    if (!e && latSide() > 0) e = dLat.reserve((size_t)B * nC * 8 * latSide() * latSide());
    if (!e && hasLos) {
      const size_t mw = (size_t)B * g.winRows * g.winCols, rw = (size_t)B * g.rWinRows * g.rWinCols;
      e = dLosVal32.reserve(mw);
      if (!e) e = dLosRt32.reserve(mw);
      if (!e && g.hasRegion) e = dRLosVal32.reserve(rw);
      if (!e && g.hasRegion) e = dRLosRt32.reserve(rw);
      const size_t nl = (size_t)nLosComps();
      losKeep = (mw + (g.hasRegion ? rw : 0)) * nl * 32 * 8 <= kLosKeepBytes;
      if (!e && losKeep) e = dLosPan.reserve(mw * nl * 64);
      if (!e && losKeep) e = dLosCnt.reserve(mw * nl);
      if (!e && losKeep && g.hasRegion) e = dRLosPan.reserve(rw * nl * 64);
      if (!e && losKeep && g.hasRegion) e = dRLosCnt.reserve(rw * nl);
    }
    if (e) return cuda_fail(e, "fast batch buffers");
    fastCap = B;
    if (graph.exec) {
      cudaGraphExecDestroy(graph.exec);
      graph = Captured{};
    }
    return 0;
  }

  static constexpr int kBoxMain = 24;  // covers radius 10 around a centre, main grid
  // CTA count of the finest launch shape (one row per CTA): bounds every shape
  // (statistic: main rows and the region's replaced rows; gradient: window rows)
  int partStride() const {
    const int los = hasLos ? kLosCtas * (fg.hasRegion ? 2 : 1) : 0;
    return std::max(fg.nDataRows + (fg.hasRegion ? fg.rRows : 0),
                    fg.winRows + (fg.hasRegion ? fg.rWinRows : 0) + los);
  }
  int boxReg() const { return fg.hasRegion ? 20 * fg.rScale + 5 : 0; }
  // the region's subsample lattice: pixels within radius 4 of a centre (every
  // pixel with the constant 20 x 20 count) lie within 4k + 1 box pixels of the
  // box centre; 20 / k lattice points per pixel step
  int latHalf() const { return 4 * fg.rScale + 1; }
  int latSide() const {
    if (!fg.hasRegion || fg.rScale < 1 || 20 % fg.rScale != 0) return 0;
    return 2 * latHalf() * (20 / fg.rScale) + 20;
  }

  // Point sources: the device descriptors carry each one's current
  // PointSource::oversamplingScale; an evaluation that computes the
  // oversampled region leaves the region's scale behind for the next one
  // (the reference's object state, core/oversampled_region.cpp:370-375).
  void syncPointSourceState() {
    if (!nPointSources || hDesc.size() != funcs.size()) return;
    bool changed = false;
    for (size_t f = 0; f < funcs.size(); f++)
      if (is_point_source(funcs[f].type) && hDesc[f].psScale != psScale[f]) {
        hDesc[f].psScale = psScale[f];
        changed = true;
      }
    if (changed)
      cudaMemcpyAsync(dDesc.p, hDesc.data(), sizeof(CompDesc) * hDesc.size(), cudaMemcpyHostToDevice, stream);
    if (!regions.empty() && !psStateFrozen)
      for (size_t f = 0; f < funcs.size(); f++)
        if (is_point_source(funcs[f].type)) psScale[f] = regions.back()->scale;
  }
  bool psStateFrozen = false;  // set while the autotuner's trial runs execute

  FastArgs fastArgs(const double *dP, double *dS, double *dG, float *modelOut) {
    syncPointSourceState();
    FastArgs a{};
    a.subTab = dSubTab.p;
    a.subBox = dSubBox.p;
    a.boxMain = kBoxMain;
    a.boxReg = boxReg();
    a.lat = latSide() > 0 ? dLat.p : nullptr;
    a.latSide = latSide();
    a.latHalf = latHalf();
    a.desc = dDesc.p;
    a.nComp = (int)funcs.size();
    a.nParams = nParamsTot;
    a.params = dP;
    a.comps = dComps32.p;
    a.bgLevel = dBg.p;
    a.data = dData32.p;
    a.weight = dW32.p;
    a.extra = (useCash && pmlr) ? dExtra32.p : nullptr;
    a.count = bootBatch ? dCountBatch.p : (doBootstrap ? dCount32.p : nullptr);
    a.countStride = bootBatch ? nDataVals : 0;
    a.dataStride = stack.n ? nDataVals : 0;
    a.entry = (stack.n || bootBatch) ? curEntry : nullptr;
    a.kind = useCash ? 1 : 0;
    a.modelErrors = modelErrors ? 1 : 0;
    a.effGain = (float)effGain;
    a.sky = (float)sky;
    a.rnTerm = (float)(nCombined * rnAduSq);
    a.psfSum = (float)psfSumFast;
    a.psfSumOs = (float)psfSumOsFast;
    a.spec = dSpec32.p;
    a.rspec = dRSpec32.p;
    a.statPart = dStatPart.p;
    a.gradPart = dGradPart.p;
    a.partStride = partStride();
    a.nStatBlocks = fast_stat_blocks(fg, tune);
    a.nGradBlocks = fast_grad_blocks(fg, tune);
    a.nRegGradBlocks = fast_reg_grad_blocks(fg, tune);
    a.stat = dS;
    a.grad = dG;
    a.done = dDone.p;
    a.modelOut = modelOut;
    a.nPs = 0;
    for (size_t f = 0; f < funcs.size() && nPointSources; f++)
      if (is_point_source(funcs[f].type)) a.psComp[a.nPs++] = (int)f;
    a.psMain = psMain32;
    a.psReg = psReg32;
    a.psPart = dPsPart.p;
    if (hasLos) {
      a.losVal = dLosVal32.p;
      a.losRt = dLosRt32.p;
      a.rLosVal = fg.hasRegion ? dRLosVal32.p : nullptr;
      a.rLosRt = fg.hasRegion ? dRLosRt32.p : nullptr;
      a.nLos = nLosComps();
      if (losKeep) {
        a.losPan = dLosPan.p;
        a.losCnt = dLosCnt.p;
        a.rLosPan = fg.hasRegion ? dRLosPan.p : nullptr;
        a.rLosCnt = fg.hasRegion ? dRLosCnt.p : nullptr;
      }
    }
    return a;
  }

  FastPlan fastPlan() {
    FastPlan p{};
    p.tune = tune;
    p.timer = timing ? &timer : nullptr;
    timer.only = timingStage.empty() ? nullptr : timingStage.c_str();
    // per-kernel timing of every stage needs them in one stream order
    if (concurrent && !(timing && timingStage.empty())) {
      p.side = side;
      p.fork0 = forkEv[0];
      p.join0 = joinEv[0];
      p.join1 = joinEv[1];
    }
    p.g = fg;
    p.Lx = &Fx;
    p.Ly = &Fy;
    p.Rx = &FRx;
    p.Ry = &FRy;
    p.H = dH32.p;
    p.Hr = dHr32.p;
    p.hPitch = even_pitch(Fx.L);
    p.hrPitch = FRx.L ? even_pitch(FRx.L) : 0;
    p.hBatch = stack.n ? (long)Fy.L * even_pitch(Fx.L) : 0;
    p.hMap = stack.n ? curEntry : nullptr;
    return p;
  }

  // Autotuner: time a few launch shapes of the row and column kernels on the
  // actual workload (the caller's parameter vectors) and keep the fastest.
  // Row shapes are tried with the automatic column shape, then column shapes
  // with the best row shape.  Runs outside any graph capture.
  int autotuneFast(int B, const double *dP, double *dS, double *dG) {
    // trial evaluations leave the point sources' state as it was
    struct Freeze {
      bool &f;
      bool old;
      explicit Freeze(bool &x) : f(x), old(x) { f = true; }
      ~Freeze() { f = old; }
    } freeze(psStateFrozen);
    const int key = B;
    auto it = tuned.find(key);
    if (it != tuned.end()) {
      tune = it->second;
      return 0;
    }
    if (stack.n && B != stack.n) {  // a subset of a stack: the whole stack's shape
      auto full = tuned.find(stack.n);
      tune = (full != tuned.end()) ? full->second : FastTune{};
      tuned[key] = tune;
      return 0;
    }
    if (hasFixedTune || !autotune) {
      tune = hasFixedTune ? fixedTune : FastTune{};
      tuned[key] = tune;
      return 0;
    }
    constexpr int kMaxSamples = 16;
    cudaEvent_t ev[2 * kMaxSamples];
    for (auto &x : ev)
      if (cudaEventCreate(&x)) return fail(IMFIT_E_CUDA, "autotune events");
    // L2-sized scratch written before each timed evaluation
    const size_t flushBytes = 256u << 20;
    void *flush = nullptr;
    if (cudaMalloc(&flush, flushBytes) != cudaSuccess) {
      cudaGetLastError();
      flush = nullptr;
    }
    const bool timingWas = timing;
    timing = false;
    auto release = [&]() {
      for (auto &x : ev) cudaEventDestroy(x);
      if (flush) cudaFree(flush);
      timing = timingWas;
    };
    // Candidates are timed on the statistic + gradient evaluation (the one a
    // fit repeats) whichever call triggers the tuning; statistic-only calls
    // use the same plan and shapes, so a parameter vector gets the same
    // statistic with or without its gradient.  Each candidate runs the way
    // later calls will: replayed from a CUDA graph when graphs are on (launch
    // costs and the programmatic-dependent overlap then match), else launched
    // kernel by kernel.  Every timed evaluation starts from an L2 cache that
    // holds none of its data (a 256 MiB write before it): a single-image
    // step's working set fits in L2, and shapes that win with warm data need
    // not win without it.  A candidate's time is the best of three trials,
    // each the sum over kSamples such evaluations, kSamples chosen so that a
    // trial holds about 2 ms of evaluations (4 to 16): the candidates differ
    // by a few percent, comparable to the noise of a single short evaluation.
    int kSamples = 4;
    auto measure = [&](const FastTune &t, float &best) -> cudaError_t {
      tune = t;
      FastArgs a = fastArgs(dP, dS, dG ? dG : dGrad.p, nullptr);
      FastPlan p = fastPlan();
      cudaGraphExec_t ex = nullptr;
      cudaError_t e = cudaSuccess;
      if (useGraphs) {
        cudaGraph_t gr;
        e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
        if (e) return e;
        cudaError_t e2 = fast_forward(p, a, B, true, stream);
        e = cudaStreamEndCapture(stream, &gr);
        if (e2) return e2;
        if (e) return e;
        e = cudaGraphInstantiate(&ex, gr, 0);
        cudaGraphDestroy(gr);
        if (e) return e;
      }
      auto run = [&]() { return ex ? cudaGraphLaunch(ex, stream) : fast_forward(p, a, B, true, stream); };
      e = run();  // warm
      best = 1e30f;
      for (int trial = 0; trial < 3 && !e; trial++) {
        for (int r = 0; r < kSamples && !e; r++) {
          if (flush) e = cudaMemsetAsync(flush, trial + r, flushBytes, stream);
          if (!e) e = cudaEventRecord(ev[2 * r], stream);
          if (!e) e = run();
          if (!e) e = cudaEventRecord(ev[2 * r + 1], stream);
        }
        if (!e) e = cudaEventSynchronize(ev[2 * kSamples - 1]);
        float sum = 0.f;
        for (int r = 0; r < kSamples && !e; r++) {
          float ms = 0.f;
          e = cudaEventElapsedTime(&ms, ev[2 * r], ev[2 * r + 1]);
          sum += ms;
        }
        best = std::min(best, sum);
      }
      if (ex) cudaGraphExecDestroy(ex);
      return e;
    };
    cudaError_t e = cudaSuccess;
    {
      float ms = 0.f;
      e = measure(FastTune{}, ms);
      if (!e && ms > 0.f)
        kSamples = std::min(kMaxSamples, std::max(4, (int)std::ceil(2.0f * (float)kSamples / ms)));
    }
    // launch shapes for the current plan: row shapes with the automatic
    // column shape, then column shapes with the best row shape
    auto tuneShapes = [&](FastTune &bestT, float &bestMs) -> cudaError_t {
      const int rowShapes[][2] = {{1, 128}, {1, 256}, {2, 256}, {3, 256}, {4, 256}, {2, 512}, {4, 512}};
      bestT = FastTune{};
      bestMs = 1e30f;
      for (auto &rs : rowShapes) {
        FastTune t{};
        t.rowRpb = rs[0];
        t.rowThreads = rs[1];
        float ms;
        cudaError_t err = measure(t, ms);
        if (err) return err;
        if (ms < bestMs) { bestMs = ms; bestT = t; }
      }
      for (int cpb : {1, 2, 4, 8}) {
        for (int nt : {0, 128, 256, 512}) {
          FastTune t = bestT;
          t.colCpb = cpb;
          t.colThreads = nt;
          float ms;
          cudaError_t err = measure(t, ms);
          if (err) return err;
          if (ms < bestMs) { bestMs = ms; bestT = t; }
        }
      }
      return cudaSuccess;
    };
    // switch to FFT plan (cand, var): a new plan re-runs the fast set-up,
    // which resizes the plan-dependent buffers (spectra) through
    // ensureFastCap here and ensureJtwjCap in the callers that need it
    auto usePlan = [&](int cand, int var) -> int {
      fftCand = cand;
      fftVariant = var;
      fastReady = false;
      int st = prepareFast();
      if (!st) st = ensureFastCap(B);
      return st;
    };
    FastTune bestT{};
    float bestMs = 1e30f;
    // the FFT plan first (padded lengths x radix orders), for a single image
    // only (image stacks keep the smallest lengths of their bucket): at the
    // first batch size, and again when a batch at least four times larger
    // arrives (a single vector leaves most SMs idle, and the plan that wins
    // there need not win on a full GPU).  Every plan is timed with the
    // default launch shape; the two fastest, if within 10 % of each other,
    // then have their launch shapes tuned and the faster tuned pair wins.
    // Plans whose default-shape times lie within the timing noise can differ
    // by several percent once their shapes are tuned.  A new plan clears the
    // launch shapes tuned for other batch sizes.
    if (!stack.n && !fftPinned && (!fftTuned || B >= 4 * fftTunedB)) {
      struct PlanTime {
        int c, v;
        float ms;
      };
      std::vector<PlanTime> plans;
      for (int cand = 0; cand < kFftCandidates && !e; cand++) {
        for (int var = 0; var < kRadixVariants && !e; var++) {
          int st = usePlan(cand, var);
          if (st) {
            release();
            return st;
          }
          float ms;
          e = measure(FastTune{}, ms);
          if (!e) plans.push_back({cand, var, ms});
        }
      }
      std::sort(plans.begin(), plans.end(), [](const PlanTime &x, const PlanTime &y) { return x.ms < y.ms; });
      size_t nFinal = 0;
      while (nFinal < plans.size() && nFinal < 2 && plans[nFinal].ms <= 1.1f * plans[0].ms) nFinal++;
      int bestC = nFinal ? plans[0].c : 0, bestV = nFinal ? plans[0].v : 0;
      for (size_t i = 0; i < nFinal && !e; i++) {
        if (nFinal > 1 || fftCand != plans[i].c || fftVariant != plans[i].v) {
          int st = usePlan(plans[i].c, plans[i].v);
          if (st) {
            release();
            return st;
          }
        }
        FastTune t;
        float ms;
        e = tuneShapes(t, ms);
        if (!e && ms < bestMs) {
          bestMs = ms;
          bestT = t;
          bestC = plans[i].c;
          bestV = plans[i].v;
        }
      }
      if (!e && (fftCand != bestC || fftVariant != bestV)) {
        int st = usePlan(bestC, bestV);
        if (st) {
          release();
          return st;
        }
      }
      fftTuned = true;
      fftTunedB = B;
    } else {
      e = tuneShapes(bestT, bestMs);
    }
    release();
    if (e) return cuda_fail(e, "autotune");
    tune = bestT;
    tuned[key] = tune;
    return 0;
  }

  // enqueue the fast evaluation for nBatch vectors already on the device
  int enqueueFast(int B, const double *dP, double *dS, double *dG, float *modelOut = nullptr) {
    int st = prepareFast();
    if (st) return st;
    if (stack.n && B != stack.n) return fail(IMFIT_E_ARG, "an image stack evaluates exactly one parameter vector per image");
    st = ensureFastCap(B);
    if (st) return st;
    st = autotuneFast(B, dP, dS, dG);  // a lookup once this (B, gradient) pair is tuned
    if (st) return st;
    const bool wantGrad = dG != nullptr;
    FastArgs a = fastArgs(dP, dS, dG ? dG : dGrad.p, modelOut);
    FastPlan p = fastPlan();
    if (useGraphs && !modelOut) {
      if (!(graph.exec && graph.nBatch == B && graph.p == dP && graph.s == dS && graph.g == dG)) {
        if (graph.exec) cudaGraphExecDestroy(graph.exec);
        graph = Captured{};
        cudaGraph_t gr;
        cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
        if (e) return cuda_fail(e, "graph capture");
        cudaError_t e2 = fast_forward(p, a, B, wantGrad, stream);
        e = cudaStreamEndCapture(stream, &gr);
        if (e2) return cuda_fail(e2, "fast path launch");
        if (e) return cuda_fail(e, "graph capture");
        e = cudaGraphInstantiate(&graph.exec, gr, 0);
        cudaGraphDestroy(gr);
        if (e) return cuda_fail(e, "graph instantiate");
        graph.nBatch = B;
        graph.p = dP;
        graph.s = dS;
        graph.g = dG;
      }
      cudaError_t e = cudaGraphLaunch(graph.exec, stream);
      if (e) return cuda_fail(e, "graph launch");
      return 0;
    }
    cudaError_t e = fast_forward(p, a, B, wantGrad, stream);
    if (e) return cuda_fail(e, "fast path launch");
    return 0;
  }

  int fastHost(int B, const double *params, double *stats, double *grads) {
    int st = prepareFast();
    if (st) return st;
    st = ensureFastCap(B);
    if (st) return st;
    const int nP = nParamsTot;
    const size_t need = (size_t)B * (2 * nP + 1);
    if (need > hMappedN) {
      if (hMapped) cudaFreeHost(hMapped);
      hMapped = dMapped = nullptr;
      hMappedN = 0;
      if (cudaHostAlloc(&hMapped, sizeof(double) * need, cudaHostAllocMapped) == cudaSuccess &&
          cudaHostGetDevicePointer(&dMapped, hMapped, 0) == cudaSuccess) {
        hMappedN = need;
      } else {
        if (hMapped) cudaFreeHost(hMapped);
        hMapped = dMapped = nullptr;
        cudaGetLastError();
      }
    }
    if (hMappedN) {  // zero-copy form
      double *hp = hMapped, *hs = hMapped + (size_t)B * nP, *hg = hs + B;
      std::copy(params, params + (size_t)B * nP, hp);
      double *dp = dMapped, *ds = dMapped + (size_t)B * nP, *dg = ds + B;
      st = enqueueFast(B, dp, ds, grads ? dg : nullptr);
      if (st) return st;
      cudaError_t e = cudaStreamSynchronize(stream);
      if (e) return cuda_fail(e, "fast results");
      std::copy(hs, hs + B, stats);
      if (grads) std::copy(hg, hg + (size_t)B * nP, grads);
      return 0;
    }
    cudaError_t e = cudaMemcpyAsync(dParams.p, params, sizeof(double) * (size_t)B * nP, cudaMemcpyHostToDevice, stream);
    if (e) return cuda_fail(e, "params upload");
    st = enqueueFast(B, dParams.p, dStat.p, grads ? dGrad.p : nullptr);
    if (st) return st;
    e = cudaMemcpyAsync(stats, dStat.p, sizeof(double) * B, cudaMemcpyDeviceToHost, stream);
    if (!e && grads) e = cudaMemcpyAsync(grads, dGrad.p, sizeof(double) * (size_t)B * nP, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "fast results");
    return 0;
  }

  // ------------------------------------------------- JtWJ (forward mode)
  int ensureJtwjCap(int B) {
    if (B <= jtwjCap) return 0;
    const FastGeom &g = fg;
    const int nP = nParamsTot, Q = nP * (nP + 1) / 2 + nP + 1;
    cudaError_t e = dModelOut.reserve((size_t)B * nDataVals);
    if (!e && nDeriv) e = dDSpec32.reserve(2 * (size_t)B * nDeriv * g.specBatch);
    if (!e && nDeriv && g.hasRegion) e = dDRSpec32.reserve(2 * (size_t)B * nDeriv * g.rSpecBatch);
    if (!e && nDeriv && g.hasRegion) e = dRegDeriv.reserve((size_t)B * nDeriv * g.rRows * g.rCols);
    if (!e) e = dJPart.reserve(2 * (size_t)B * Q * partStride());  // (hi, lo) pairs
    if (!e) e = dAlpha.reserve((size_t)B * nP * nP);
    if (!e) e = dBeta.reserve((size_t)B * nP);
    if (e) return cuda_fail(e, "JtWJ buffers");
    jtwjCap = B;
    return 0;
  }

  // statistic, J^T J and J^T dev for B parameter vectors on the device
  // (jacOut, optional: [B][nP + 1][nData] FP32 Jacobian columns and deviates)
  int enqueueJtwj(int B, const double *dP, double *dS, double *dA, double *dBt, float *jacOut = nullptr) {
    int st = prepareFast();
    if (st) return st;
    if (useCash && !pmlr)
      return fail(IMFIT_E_UNSUPPORTED, "J^T J needs per-pixel deviates: chi^2 or Poisson-MLR, not the Cash statistic");
    if (hasLos)
      return fail(IMFIT_E_UNSUPPORTED, "J^T J of 3-D line-of-sight components is not available; use the adjoint "
                                       "gradient (imfit_GetFitStatisticAndGradient)");
    if (stack.n && (curEntry ? B > stack.n : B != stack.n))
      return fail(IMFIT_E_ARG, "an image stack evaluates exactly one parameter vector per image");
    st = ensureFastCap(B);
    if (st) return st;
    if (!dP || !dS || !dA || !dBt) return fail(IMFIT_E_ARG, "JtWJ: null device buffer");
    st = autotuneFast(B, dP, dS, nullptr);
    if (st) return st;
    // after the autotuner: its choice of FFT plan sets the derivative spectra's size
    st = ensureJtwjCap(B);
    if (st) return st;
    FastArgs a = fastArgs(dP, dS, dGrad.p, dModelOut.p);
    FastPlan p = fastPlan();
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (fast_jtwj_smem(p, nDeriv, nParamsTot) > (size_t)optin)
      return fail(IMFIT_E_UNSUPPORTED, "J^T J: too many parameters for this image width (shared memory)");
    JtwjArgs J{};
    J.dspec = dDSpec32.p;
    J.drspec = dDRSpec32.p;
    J.regDeriv = dRegDeriv.p;
    J.slot = dSlot.p;
    J.nD = nDeriv;
    J.part = reinterpret_cast<float2 *>(dJPart.p);
    J.alpha = dA;
    J.beta = dBt;
    J.stat = dS;
    J.jac = jacOut;
    cudaError_t e = fast_jtwj(p, a, J, B, stream);
    if (e) return cuda_fail(e, "JtWJ launch");
    return 0;
  }

  // imageMap (host, B entries; image stacks only): batch entry b fits image imageMap[b]
  int jtwjHost(int B, const double *params, double *stats, double *alpha, double *beta,
               const int *imageMap = nullptr) {
    int st = prepareFast();
    if (!st) st = ensureFastCap(B);
    // the output buffers must exist before their addresses are taken below
    if (!st) st = ensureJtwjCap(B);
    if (st) return st;
    curEntry = nullptr;
    const int nEntries = stack.n ? stack.n : bootBatch;
    if (imageMap && nEntries) {
      for (int i = 0; i < B; i++)
        if (imageMap[i] < 0 || imageMap[i] >= nEntries) return fail(IMFIT_E_ARG, "image index out of range");
      cudaError_t e0 = dEntry.reserve(B);
      if (!e0) e0 = cudaMemcpyAsync(dEntry.p, imageMap, sizeof(int) * B, cudaMemcpyHostToDevice, stream);
      if (e0) return cuda_fail(e0, "image map upload");
      curEntry = dEntry.p;
    }
    const int nP = nParamsTot;
    cudaError_t e = cudaMemcpyAsync(dParams.p, params, sizeof(double) * (size_t)B * nP, cudaMemcpyHostToDevice, stream);
    if (e) return cuda_fail(e, "params upload");
    st = enqueueJtwj(B, dParams.p, dStat.p, dAlpha.p, dBeta.p);
    curEntry = nullptr;
    if (st) return st;
    e = cudaMemcpyAsync(stats, dStat.p, sizeof(double) * B, cudaMemcpyDeviceToHost, stream);
    if (!e && alpha) e = cudaMemcpyAsync(alpha, dAlpha.p, sizeof(double) * (size_t)B * nP * nP, cudaMemcpyDeviceToHost, stream);
    if (!e && beta) e = cudaMemcpyAsync(beta, dBeta.p, sizeof(double) * (size_t)B * nP, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "JtWJ results");
    return 0;
  }

  // Image stack: nImg images of nc x nr pixels, per-pixel sigmas (internal
  // weight 1/sigma as AddErrorVector with WEIGHTS_ARE_SIGMAS; sigma <= 0 or
  // non-finite masks the pixel, as does a non-finite data value) and one PSF
  // per image, normalised with the Convolver's Kahan sum.  chi^2 statistic.
  int setupStack(int nImg, int nc, int nr, const double *img, const double *sigma, const double *psfs, int pc,
                 int pr) {
    if (!setsDefined) return fail(IMFIT_E_STATE, "DefineFunctionSets not called");
    if (nImg < 1 || nc < 1 || nr < 1 || pc < 1 || pr < 1 || !img || !sigma || !psfs)
      return fail(IMFIT_E_ARG, "bad image stack arguments");
    if (dataValsSet) return fail(IMFIT_E_STATE, "image data already added to this ModelObject");
    if (useCash || doBootstrap) return fail(IMFIT_E_UNSUPPORTED, "image stacks use the chi^2 statistic");
    const long n = (long)nc * nr;
    stack = Stack{};
    stack.n = nImg;
    stack.pc = pc;
    stack.pr = pr;
    stack.data.resize((size_t)n * nImg);
    stack.weight.resize((size_t)n * nImg);
    for (size_t z = 0; z < stack.data.size(); z++) {
      const double d = img[z], sg = sigma[z];
      const bool good = std::isfinite(d) && std::isfinite(sg) && sg > 0.0;
      stack.data[z] = good ? (float)d : 0.f;
      stack.weight[z] = good ? (float)(1.0 / sg) : 0.f;
    }
    const long np = (long)pc * pr;
    stack.psf.assign(psfs, psfs + np * nImg);
    for (int i = 0; i < nImg; i++) {
      double *q = stack.psf.data() + (size_t)i * np;
      for (long k = 0; k < np; k++)
        if (!std::isfinite(q[k])) return fail(IMFIT_E_ARG, "PSF image has one or more non-finite values");
      const double ks = kahan_sum(q, np);
      if (!(ks > 0.0)) return fail(IMFIT_E_ARG, "Sum of PSF pixel values is <= 0 -- PSF cannot be normalized");
      for (long k = 0; k < np; k++) q[k] = q[k] / ks;
    }
    nDataCols = nc;
    nDataRows = nr;
    nDataVals = n;
    nValid = n;
    doConv = true;
    nPsfCols = pc;
    nPsfRows = pr;
    finalSetupDone = true;
    fastReady = false;
    return 0;
  }

  // ---------------------------------------------------- ragged cutout sets
  // nImg cutouts: cutout i has cols[i] x rows[i] pixels (data and sigma
  // concatenated row-major, cutout after cutout) and a pcols[i] x prows[i]
  // PSF (odd sizes, concatenated; normalised here with a Kahan sum).  Pixels
  // with a non-finite value or sigma <= 0 are masked.  chi^2 with the given
  // sigmas; the model's functions must be pixel functions (no 3-D or point
  // sources) and the handle may hold no image of its own.
  int setupCutouts(int nImg, const int *cols, const int *rows, const double *img, const double *sigma,
                   const int *pcols, const int *prows, const double *psfs) {
    if (!setsDefined) return fail(IMFIT_E_STATE, "DefineFunctionSets not called");
    if (nImg < 1 || !cols || !rows || !img || !sigma || !pcols || !prows || !psfs)
      return fail(IMFIT_E_ARG, "bad cutout-set arguments");
    if (dataValsSet || stack.n || rag.n) return fail(IMFIT_E_STATE, "image data already added to this ModelObject");
    if (!regions.empty() || useCash || doBootstrap) return fail(IMFIT_E_UNSUPPORTED, "cutout sets use chi^2 only");
    for (auto &f : funcs)
      if (is_los(f.type) || is_point_source(f.type))
        return fail(IMFIT_E_UNSUPPORTED, "cutout sets take pixel functions only (no 3-D or point sources)");
    if ((int)funcs.size() > kMaxComponents) return fail(IMFIT_E_UNSUPPORTED, "too many components");
    RagSet &R = rag;
    R.ent.assign(nImg, RagEntry{});
    R.totalPix = R.totalSpec = R.totalRows = 0;
    R.maxM = R.maxLy = R.maxCols = 0;
    std::vector<long> psfOff(nImg);
    long np = 0;
    for (int i = 0; i < nImg; i++) {
      const int nc = cols[i], nr = rows[i], pc = pcols[i], pr = prows[i];
      if (nc < 1 || nr < 1 || pc < 1 || pr < 1 || !(pc & 1) || !(pr & 1))
        return fail(IMFIT_E_ARG, "cutout sizes must be positive and PSF sizes odd");
      psfOff[i] = np;
      np += (long)pc * pr;
      RagEntry &E = R.ent[i];
      E.nDataCols = nc;
      E.nDataRows = nr;
      E.winCols = nc + pc - 1;
      E.winRows = nr + pr - 1;
      E.xOrig = 2 - pc + pc / 2;
      E.yOrig = 2 - pr + pr / 2;
      E.Lx = smooth_size(E.winCols, true);
      E.Ly = smooth_size(E.winRows, true);
      if (E.Lx / 2 > 4096 || E.Ly > 4096) return fail(IMFIT_E_UNSUPPORTED, "cutout too large for the fast path");
      E.pitch = even_pitch(E.Lx);
      E.colGroups = (E.Lx / 2 + 1 + kRagColsPerCta - 1) / kRagColsPerCta;
      E.specSize = (long)E.Ly * E.pitch;
      E.specOff = R.totalSpec;
      E.hOff = R.totalSpec;  // one PSF spectrum per cutout, same geometry
      E.dataOff = R.totalPix;
      E.rowOff = R.totalRows;
      R.totalPix += (long)nc * nr;
      R.totalSpec += E.specSize;
      R.totalRows += nr;
      R.maxM = std::max(R.maxM, E.Lx / 2);
      R.maxLy = std::max(R.maxLy, E.Ly);
      R.maxCols = std::max(R.maxCols, nc);
    }
    R.totalH = R.totalSpec;
    // FFT tables per distinct length
    auto table = [&](int L) -> FFTLen * {
      auto it = R.lens.find(L);
      if (it != R.lens.end()) return it->second.get();
      std::unique_ptr<FFTLen> t(new FFTLen());
      if (fftlen_create(*t, L)) return nullptr;
      FFTLen *raw = t.get();
      R.lens[L] = std::move(t);
      return raw;
    };
    auto plan = [](const FFTTable &t) {
      FFTPlan<float> p;
      p.n = t.n;
      p.npass = t.npass;
      p.radix = pack_radix(t.radix, t.npass);
      p.tw = reinterpret_cast<const cplx<float> *>(t.tw32);
      p.padFirst = fft_pad_enabled() && fft_pad_first(p.npass, p.radix);
      return p;
    };
    // data, weights, PSF spectra
    std::vector<float> d32(R.totalPix), w32(R.totalPix);
    for (long z = 0; z < R.totalPix; z++) {
      const double d = img[z], sg = sigma[z];
      const bool good = std::isfinite(d) && std::isfinite(sg) && sg > 0.0;
      d32[z] = good ? (float)d : 0.f;
      w32[z] = good ? (float)(1.0 / sg) : 0.f;
    }
    cudaError_t e = dRagData.reserve(R.totalPix);
    if (!e) e = dRagW.reserve(R.totalPix);
    if (!e) e = cudaMemcpy(dRagData.p, d32.data(), sizeof(float) * R.totalPix, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(dRagW.p, w32.data(), sizeof(float) * R.totalPix, cudaMemcpyHostToDevice);
    if (!e) e = dRagH.reserve(2 * (size_t)R.totalH);
    if (e) return cuda_fail(e, "cutout-set buffers");
    for (int i = 0; i < nImg; i++) {
      RagEntry &E = R.ent[i];
      const int pc = pcols[i], pr = prows[i];
      std::vector<double> q(psfs + psfOff[i], psfs + psfOff[i] + (long)pc * pr);
      for (double v : q)
        if (!std::isfinite(v)) return fail(IMFIT_E_ARG, "PSF image has one or more non-finite values");
      const double ks = kahan_sum(q.data(), (long)q.size());
      if (!(ks > 0.0)) return fail(IMFIT_E_ARG, "Sum of PSF pixel values is <= 0 -- PSF cannot be normalized");
      for (double &v : q) v = v / ks;
      FFTLen *fx = table(E.Lx), *fy = table(E.Ly);
      if (!fx || !fy) return fail(IMFIT_E_CUDA, "FFT tables");
      int st = shiftedSpectrum32To(q.data(), pc, pr, *fx, *fy, dRagH.p + 2 * E.hOff);
      if (st) return st;
      E.rowPlan = plan(fx->half);
      E.colPlan = plan(fy->full);
      E.colPlanI = plan(fy->fullRev);
      if (E.colPlan.npass < 2) E.colPlanI.tw = nullptr;  // a single pass: the unfused column group
      E.twL = reinterpret_cast<const cplx<float> *>(fx->twL32);
    }
    e = dRagEnt.reserve(nImg);
    if (!e) e = cudaMemcpy(dRagEnt.p, R.ent.data(), sizeof(RagEntry) * nImg, cudaMemcpyHostToDevice);
    // component descriptors and derivative slots (every parameter but constant backgrounds)
    std::vector<CompDesc> desc(funcs.size());
    for (size_t f = 0; f < funcs.size(); f++) {
      CompDesc &dd = desc[f];
      dd = CompDesc{};
      dd.type = funcs[f].type;
      dd.subsample = funcs[f].subsample;
      dd.paramOffset = paramOffset[f];
      dd.x0Index = x0Index[f];
      dd.nParams = funcs[f].nParams;
      dd.background = (funcs[f].type == F_FLATSKY) ? 1 : 0;
    }
    hRagSlot.assign(nParamsTot, 0);
    for (auto &dd : desc)
      if (dd.background) hRagSlot[dd.paramOffset] = -1;
    ragNDeriv = 0;
    for (int j = 0; j < nParamsTot; j++)
      if (hRagSlot[j] >= 0) hRagSlot[j] = ragNDeriv++;
    if (!e) e = dRagDesc.reserve(desc.size());
    if (!e) e = cudaMemcpy(dRagDesc.p, desc.data(), sizeof(CompDesc) * desc.size(), cudaMemcpyHostToDevice);
    if (!e) e = dRagSlot.reserve(std::max(nParamsTot, 1));
    if (!e) e = cudaMemcpy(dRagSlot.p, hRagSlot.data(), sizeof(int) * nParamsTot, cudaMemcpyHostToDevice);
    // evaluation buffers, sized for all cutouts active
    const int nP = nParamsTot, nC = (int)funcs.size(), Q = nP * (nP + 1) / 2 + nP + 1;
    if (!e) e = dRagSpec.reserve(2 * (size_t)R.totalSpec);
    if (!e && ragNDeriv) e = dRagDSpec.reserve(2 * (size_t)ragNDeriv * R.totalSpec);
    if (!e) e = dRagModel.reserve(R.totalPix);
    if (!e) e = dRagPart.reserve(2 * (size_t)Q * R.totalRows);  // (hi, lo) pairs
    if (!e) e = dRagParams.reserve((size_t)nImg * nP);
    if (!e) e = dRagS.reserve(nImg);
    if (!e) e = dRagA.reserve((size_t)nImg * nP * nP);
    if (!e) e = dRagB.reserve((size_t)nImg * nP);
    if (!e) e = dRagComps.reserve((size_t)nImg * nC);
    if (!e) e = dRagBg.reserve(2 * (size_t)nImg);
    if (!e) e = dRagSubTab.reserve((size_t)nImg * nC * kBoxMain * kBoxMain * 8);
    if (!e) e = dRagSubBox.reserve((size_t)nImg * nC * 4);
    if (!e) e = dRagWork.reserve((size_t)(kRagWorkKinds + 1) * (nImg + 1));
    if (e) return cuda_fail(e, "cutout-set buffers");
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (rag_jtwj_smem(R.maxM, ragNDeriv, nParamsTot, R.maxCols) > (size_t)optin)
      return fail(IMFIT_E_UNSUPPORTED, "cutout set: the largest cutout needs more shared memory than a CTA has");
    R.n = nImg;
    nValid = R.totalPix;
    finalSetupDone = true;
    return 0;
  }

  // statistic, J^T J and J^T dev of the cutouts entries[0..K) at params (K x nP, host)
  int ragJtwjHost(int K, const int *entries, const double *params, double *stats, double *alpha, double *beta) {
    if (!rag.n) return fail(IMFIT_E_STATE, "no cutout set (imfit_SetupCutouts)");
    if (K < 1 || K > rag.n || !entries || !params || !stats || !alpha || !beta)
      return fail(IMFIT_E_ARG, "bad cutout-set J^T J arguments");
    RagSet &R = rag;
    const int nP = nParamsTot;
    // work lists: act, then per kind the prefix sums of the slots' counts
    std::vector<int> &w = R.work;
    w.assign((size_t)(kRagWorkKinds + 1) * (K + 1), 0);
    int *act = w.data();
    int *pre[kRagWorkKinds];
    for (int t = 0; t < kRagWorkKinds; t++) pre[t] = w.data() + (size_t)(t + 1) * (K + 1);
    for (int k = 0; k < K; k++) {
      const int en = entries[k];
      if (en < 0 || en >= R.n) return fail(IMFIT_E_ARG, "cutout index out of range");
      act[k] = en;
      const RagEntry &E = R.ent[en];
      pre[kRagWinRows][k + 1] = pre[kRagWinRows][k] + E.winRows;
      pre[kRagDataRows][k + 1] = pre[kRagDataRows][k] + E.nDataRows;
      pre[kRagCols][k + 1] = pre[kRagCols][k] + E.colGroups;
      pre[kRagDerivCols][k + 1] = pre[kRagDerivCols][k] + E.colGroups * ragNDeriv;
    }
    cudaError_t e = cudaMemcpyAsync(dRagWork.p, w.data(), sizeof(int) * w.size(), cudaMemcpyHostToDevice, stream);
    if (!e)
      e = cudaMemcpyAsync(dRagParams.p, params, sizeof(double) * (size_t)K * nP, cudaMemcpyHostToDevice, stream);
    if (e) return cuda_fail(e, "cutout-set upload");
    FastArgs a{};
    a.desc = dRagDesc.p;
    a.nComp = (int)funcs.size();
    a.nParams = nP;
    a.params = dRagParams.p;
    a.comps = dRagComps.p;
    a.bgLevel = dRagBg.p;
    a.data = dRagData.p;
    a.weight = dRagW.p;
    a.kind = 0;
    a.effGain = 1.f;
    a.psfSum = 1.f;
    a.psfSumOs = 1.f;
    a.subTab = dRagSubTab.p;
    a.subBox = dRagSubBox.p;
    a.boxMain = kBoxMain;
    a.boxReg = 0;
    RagArgs r{};
    r.ent = dRagEnt.p;
    r.act = dRagWork.p;
    r.K = K;
    r.lines = 1;
    r.spec = reinterpret_cast<cplx<float> *>(dRagSpec.p);
    r.H = reinterpret_cast<const cplx<float> *>(dRagH.p);
    r.model = dRagModel.p;
    r.part = reinterpret_cast<float2 *>(dRagPart.p);
    r.totalRows = R.totalRows;
    const int *starts[kRagWorkKinds];
    int totals[kRagWorkKinds];
    for (int t = 0; t < kRagWorkKinds; t++) {
      starts[t] = dRagWork.p + (size_t)(t + 1) * (K + 1);
      totals[t] = pre[t][K];
    }
    r.start = starts[kRagWinRows];
    e = rag_jtwj(a, r, reinterpret_cast<cplx<float> *>(dRagDSpec.p), starts, totals, dRagSlot.p, ragNDeriv, R.maxM,
                 R.maxLy, R.maxCols, dRagA.p, dRagB.p, dRagS.p, stream);
    if (e) return cuda_fail(e, "cutout-set J^T J launch");
    e = cudaMemcpyAsync(stats, dRagS.p, sizeof(double) * K, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaMemcpyAsync(alpha, dRagA.p, sizeof(double) * (size_t)K * nP * nP, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaMemcpyAsync(beta, dRagB.p, sizeof(double) * (size_t)K * nP, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "cutout-set J^T J results");
    return 0;
  }

  struct LMBatchStats {
    int rounds = 0;          // J^T W J evaluations (rounds of the lockstep LM, the first included)
    long evaluations = 0;    // problem evaluations over all rounds
    double evalSeconds = 0;  // wall time inside them
    double totalSeconds = 0;
  } lmStats;

  int fitLMBatch(int B, double *params, const int *fixed, const double *lower, const double *upper, double ftol,
                 int maxIter, double *stats, int *nIter, int *status) {
    const int n = nParamsTot;
    if (rag.n && B != rag.n) return fail(IMFIT_E_ARG, "a cutout set fits exactly one parameter vector per cutout");
    LMSettings set;
    set.ftol = ftol;
    if (maxIter > 0) set.maxIter = maxIter;
    std::vector<double> hA((size_t)B * n * n), hB((size_t)B * n);
    // evaluate only the problems still running (compacted; on a stack each
    // keeps its own image through the image map)
    std::vector<int> idx;
    std::vector<double> Xs, Ss, As, Bs;
    JtwjBatchEval ev = [&, this](const double *X, const unsigned char *act, double *S, double *A, double *b) {
      idx.clear();
      for (int i = 0; i < B; i++)
        if (act[i]) idx.push_back(i);
      const int k = (int)idx.size();
      if (k == 0) return 0;
      if (rag.n) {  // cutout set: one launch per stage over the active cutouts
        Xs.resize((size_t)k * n);
        Ss.resize(k);
        As.resize((size_t)k * n * n);
        Bs.resize((size_t)k * n);
        for (int r = 0; r < k; r++)
          std::copy(X + (size_t)idx[r] * n, X + (size_t)(idx[r] + 1) * n, Xs.begin() + (size_t)r * n);
        int st = ragJtwjHost(k, idx.data(), Xs.data(), Ss.data(), As.data(), Bs.data());
        if (st) return st;
        for (int r = 0; r < k; r++) {
          const int i = idx[r];
          S[i] = Ss[r];
          std::copy(As.begin() + (size_t)r * n * n, As.begin() + (size_t)(r + 1) * n * n, A + (size_t)i * n * n);
          std::copy(Bs.begin() + (size_t)r * n, Bs.begin() + (size_t)(r + 1) * n, b + (size_t)i * n);
        }
        return 0;
      }
      if (k == B) return jtwjHost(B, X, S, A, b);
      Xs.resize((size_t)k * n);
      Ss.resize(k);
      As.resize((size_t)k * n * n);
      Bs.resize((size_t)k * n);
      for (int r = 0; r < k; r++)
        std::copy(X + (size_t)idx[r] * n, X + (size_t)(idx[r] + 1) * n, Xs.begin() + (size_t)r * n);
      int st = jtwjHost(k, Xs.data(), Ss.data(), As.data(), Bs.data(), (stack.n || bootBatch) ? idx.data() : nullptr);
      if (st) return st;
      for (int r = 0; r < k; r++) {
        const int i = idx[r];
        S[i] = Ss[r];
        std::copy(As.begin() + (size_t)r * n * n, As.begin() + (size_t)(r + 1) * n * n, A + (size_t)i * n * n);
        std::copy(Bs.begin() + (size_t)r * n, Bs.begin() + (size_t)(r + 1) * n, b + (size_t)i * n);
      }
      return 0;
    };
    std::vector<LMResult> res(B);
    // where the time goes: the J^T W J evaluations (device work and transfers)
    // and the rest (the host's LM steps)
    lmStats = LMBatchStats{};
    JtwjBatchEval timed = [&](const double *X, const unsigned char *act, double *S, double *A, double *b) {
      const auto t0 = std::chrono::steady_clock::now();
      const int r = ev(X, act, S, A, b);
      lmStats.evalSeconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      lmStats.rounds++;
      for (int i = 0; i < B; i++) lmStats.evaluations += act[i] ? 1 : 0;
      return r;
    };
    const auto t0 = std::chrono::steady_clock::now();
    int st = lm_minimize_batch(B, n, params, fixed, lower, upper, set, timed, res.data());
    lmStats.totalSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (int i = 0; i < B; i++) {
      if (stats) stats[i] = res[i].stat;
      if (nIter) nIter[i] = res[i].nIter;
      if (status) status[i] = res[i].status;
    }
    return st < 0 ? st : 0;
  }

  // Jacobian of the deviates (mpfit's derivative vectors for side = 3,
  // solvers/mpfit.cpp:1210-1232): column j of fjac (nDataVals values) is
  // d dev / d param_j, FP32-evaluated, in the order ComputeDeviates writes.
  int jacobianHost(const double *params, double *fjac, double *deviates) {
    int st = prepareFast();
    if (st) return st;
    if (doBootstrap) return fail(IMFIT_E_UNSUPPORTED, "the Jacobian is per data pixel; not with a bootstrap sample");
    if (stack.n) return fail(IMFIT_E_UNSUPPORTED, "the Jacobian is per image; use a single-image ModelObject");
    st = ensureFastCap(1);
    if (!st) st = ensureJtwjCap(1);
    if (st) return st;
    const int nP = nParamsTot;
    DevBuf<float> jac;
    cudaError_t e = jac.reserve((size_t)(nP + 1) * nDataVals);
    if (!e) e = cudaMemcpyAsync(dParams.p, params, sizeof(double) * nP, cudaMemcpyHostToDevice, stream);
    if (e) return cuda_fail(e, "Jacobian buffers");
    curEntry = nullptr;
    st = enqueueJtwj(1, dParams.p, dStat.p, dAlpha.p, dBeta.p, jac.p);
    if (st) return st;
    std::vector<float> h((size_t)(nP + 1) * nDataVals);
    e = cudaMemcpyAsync(h.data(), jac.p, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "Jacobian results");
    for (size_t k = 0; k < (size_t)nP * nDataVals; k++) fjac[k] = h[k];
    if (deviates)
      for (long z = 0; z < nDataVals; z++) deviates[z] = h[(size_t)nP * nDataVals + z];
    return 0;
  }

  // ModelObject::MakeBootstrapSample (core/model_object.cpp:2061-2087): nValid
  // draws of a data index by genrand_real2, rejecting pixels of weight <= 0
  void drawBootstrap(std::vector<long> &idx) {
    idx.assign(nValid, 0);
    for (long i = 0; i < nValid; i++) {
      long n;
      do {
        n = (long)floor(rng.real2() * nDataVals);
      } while (!(weight[n] > 0.0));
      idx[i] = n;
    }
  }

  // K bootstrap refits at once (core/bootstrap_errors.cpp:160-240 runs them one
  // after another): the next K samples of the MT19937 stream, each held as
  // per-pixel multiplicities, fitted from bestfit by the lockstep batched LM.
  int bootstrapFitBatch(int K, const double *bestfit, const int *fixed, const double *lower, const double *upper,
                        double ftol, int maxIter, double *params, double *stats, int *nIter, int *status) {
    if (!doBootstrap) return fail(IMFIT_E_STATE, "UseBootstrap not called");
    if (stack.n) return fail(IMFIT_E_UNSUPPORTED, "bootstrap refits of an image stack");
    if (K < 1 || !bestfit || !params) return fail(IMFIT_E_ARG, "bad bootstrap batch arguments");
    int st = prepareFast();
    if (st) return st;
    std::vector<float> cnt((size_t)K * nDataVals, 0.f);
    for (int k = 0; k < K; k++) {
      drawBootstrap(bootIdx);
      float *c = cnt.data() + (size_t)k * nDataVals;
      for (long i = 0; i < nValid; i++) c[bootIdx[i]] += 1.f;
    }
    // the last sample drawn stays the handle's current one, as after the reference's loop
    st = uploadBootstrap();
    if (st) return st;
    cudaError_t e = dCountBatch.reserve(cnt.size());
    if (!e) e = cudaMemcpy(dCountBatch.p, cnt.data(), sizeof(float) * cnt.size(), cudaMemcpyHostToDevice);
    if (e) return cuda_fail(e, "bootstrap multiplicities");
    const int n = nParamsTot;
    for (int k = 0; k < K; k++) std::copy(bestfit, bestfit + n, params + (size_t)k * n);
    std::vector<double> lo, hi;
    if (lower) {
      lo.resize((size_t)K * n);
      for (int k = 0; k < K; k++) std::copy(lower, lower + n, lo.begin() + (size_t)k * n);
    }
    if (upper) {
      hi.resize((size_t)K * n);
      for (int k = 0; k < K; k++) std::copy(upper, upper + n, hi.begin() + (size_t)k * n);
    }
    dropGraph();
    bootBatch = K;
    st = fitLMBatch(K, params, fixed, lower ? lo.data() : nullptr, upper ? hi.data() : nullptr, ftol, maxIter,
                    stats, nIter, status);
    bootBatch = 0;
    dropGraph();
    return st;
  }

  void dropGraph() {
    if (graph.exec) cudaGraphExecDestroy(graph.exec);
    graph = Captured{};
  }

  int makeBootstrapSample() {
    if (!finalSetupDone) return fail(IMFIT_E_STATE, "FinalSetupForFitting not called");
    drawBootstrap(bootIdx);
    return uploadBootstrap();
  }

  int uploadBootstrap() {
    cudaError_t e = dBoot.reserve(nValid);
    if (!e) e = cudaMemcpy(dBoot.p, bootIdx.data(), sizeof(long) * nValid, cudaMemcpyHostToDevice);
    if (!e && fastReady) e = uploadCounts();
    if (e) return cuda_fail(e, "bootstrap indices");
    return 0;
  }
};

static thread_local std::string g_createError;

namespace imfit {
// message for imfit_LastError(NULL) from entry points that take no handle
void set_global_error(const char *msg) { g_createError = msg ? msg : ""; }
}  // namespace imfit

#define GET(m)                                                     \
  if (!(m)) return IMFIT_E_ARG;                                    \
  if (cudaSetDevice((m)->device) != cudaSuccess) return IMFIT_E_CUDA;

extern "C" {

const char *imfit_Version(void) { return kVersion; }

int imfit_ModelObject_new(int device, imfit_model_t *out) {
  if (!out) return IMFIT_E_ARG;
  *out = nullptr;
  cudaError_t e = cudaSetDevice(device);
  if (e) {
    g_createError = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return IMFIT_E_CUDA;
  }
  auto *m = new imfit_model_s();
  m->device = device;
  e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  // the oversampled region's pipeline (side stream) finishes last when both
  // windows' passes share the SMs: its CTAs go first
  int prioLeast = 0, prioGreatest = 0;
  if (!e) e = cudaDeviceGetStreamPriorityRange(&prioLeast, &prioGreatest);
  if (!e) e = cudaStreamCreateWithPriority(&m->side, cudaStreamNonBlocking, prioGreatest);

  for (int i = 0; i < 2 && !e; i++) {
    e = cudaEventCreateWithFlags(&m->forkEv[i], cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&m->joinEv[i], cudaEventDisableTiming);
  }
  if (e) {
    g_createError = std::string("stream/event creation: ") + cudaGetErrorString(e);
    delete m;
    return IMFIT_E_CUDA;
  }
  // kernel attributes are set once here, before any stream capture can begin
  fast_prepare_kernels();
  fft_prepare_kernels();
  *out = m;
  return 0;
}

int imfit_ModelObject_delete(imfit_model_t m) {
  if (!m) return 0;
  cudaSetDevice(m->device);
  cudaStreamSynchronize(m->stream);
  delete m;
  return 0;
}

const char *imfit_LastError(imfit_model_t m) { return m ? m->lastError.c_str() : g_createError.c_str(); }

int imfit_AddFunction(imfit_model_t m, const char *name) {
  GET(m);
  if (!name) return m->fail(IMFIT_E_ARG, "null function name");
  FuncInfo f;
  if (!lookup_function(name, f)) return m->fail(IMFIT_E_UNSUPPORTED, std::string("unknown or unsupported function: ") + name);
  if (m->funcs.size() >= (size_t)kMaxComponents) return m->fail(IMFIT_E_UNSUPPORTED, "too many functions");
  m->funcs.push_back(f);
  m->psScale.push_back(1);
  if (is_point_source(f.type)) {
    m->nPointSources++;
    m->psKind = 0;
  }
  m->setsDefined = false;
  return 0;
}

int imfit_SetFunctionOptionalParam(imfit_model_t m, int i, const char *name, const char *value) {
  GET(m);
  if (i < 0 || i >= (int)m->funcs.size() || !name || !value) return m->fail(IMFIT_E_ARG, "bad function index or name");
  FuncInfo &f = m->funcs[i];
  if (!is_point_source(f.type))
    return m->fail(IMFIT_E_UNSUPPORTED, f.name + " takes no optional parameters");
  if (std::string(name) != "method") return m->fail(IMFIT_E_ARG, std::string("unrecognized optional parameter ") + name);
  const std::string v(value);
  int kind = 0;
  if (v == "bicubic" || v == "Bicubic") kind = PSF_BICUBIC;
  if (v == "lanczos2" || v == "Lanczos2") kind = PSF_LANCZOS2;
  if ((v == "lanczos3" || v == "Lanczos3") && f.type == F_POINTSOURCE) kind = PSF_LANCZOS3;
  if (!kind) return m->fail(IMFIT_E_ARG, "unidentified interpolation type " + v);
  f.method = kind;
  m->psKind = 0;
  m->fastReady = false;
  return 0;
}

int imfit_SetSubsampling(imfit_model_t m, int i, int s) {
  GET(m);
  if (i < 0 || i >= (int)m->funcs.size()) return m->fail(IMFIT_E_ARG, "bad function index");
  m->funcs[i].subsample = s ? 1 : 0;
  m->fastReady = false;
  return 0;
}

int imfit_DefineFunctionSets(imfit_model_t m, const int *starts, int n) {
  GET(m);
  if (n < 0 || (n > 0 && !starts)) return m->fail(IMFIT_E_ARG, "bad function-set list");
  return m->defineSets(starts, n);
}

int imfit_PopulateParameterNames(imfit_model_t m) {
  GET(m);
  if (!m->setsDefined) return m->fail(IMFIT_E_STATE, "DefineFunctionSets not called");
  m->populateNames();
  return 0;
}

int imfit_GetParameterName(imfit_model_t m, int i, char *buf, int len) {
  GET(m);
  if (!buf || len < 1) return IMFIT_E_ARG;
  const char *s = (i >= 0 && i < (int)m->paramNames.size()) ? m->paramNames[i].c_str() : "<undefined>";
  snprintf(buf, len, "%s", s);
  return 0;
}

int imfit_AddPSFVector(imfit_model_t m, long nPix, int nc, int nr, const double *psf, int normalize) {
  GET(m);
  if (!psf || nc < 1 || nr < 1 || nPix != (long)nc * nr) return m->fail(IMFIT_E_ARG, "bad PSF arguments");
  double s = 0.0;
  for (long i = 0; i < nPix; i++) {
    if (!std::isfinite(psf[i])) return m->fail(-1, "PSF image has one or more non-finite values");
    s += psf[i];
  }
  if (normalize && s <= 0.0) return m->fail(-1, "Sum of PSF pixel values is <= 0 -- PSF cannot be normalized");
  m->psf.assign(psf, psf + nPix);
  if (normalize) {
    const double ks = kahan_sum(m->psf.data(), nPix);
    for (auto &v : m->psf) v = v / ks;
  }
  m->psfSum = 0.0;
  for (double v : m->psf) m->psfSum += v;
  m->nPsfCols = nc;
  m->nPsfRows = nr;
  m->doConv = true;
  m->psfNormalize = normalize != 0;
  m->psKind = 0;  // point-source interpolator rebuilt from this PSF
  if (m->modelSetupDone) return m->fail(-1, "PSF was added after SetupModelImage() was already called");
  return 0;
}

int imfit_SetupModelImage(imfit_model_t m, int nc, int nr) {
  GET(m);
  return m->setupModelImage(nc, nr);
}

int imfit_AddImageDataVector(imfit_model_t m, const double *pix, int nc, int nr) {
  GET(m);
  if (!pix || nc < 1 || nr < 1) return m->fail(IMFIT_E_ARG, "bad image");
  m->data.assign(pix, pix + (size_t)nc * nr);
  m->nDataVals = m->nValid = (long)nc * nr;
  m->dataValsSet = true;
  int st = m->setupModelImage(nc, nr);
  return st ? -1 : 0;
}

int imfit_AddImageCharacteristics(imfit_model_t m, double gain, double rn, double texp, int ncomb, double sky) {
  GET(m);
  if (!(gain > 0.0) || rn < 0.0 || !(texp > 0.0) || ncomb < 1 || sky < 0.0)
    return m->fail(IMFIT_E_ARG, "bad image characteristics");
  m->gain = gain;
  m->readNoise = rn;
  m->expTime = texp;
  m->nCombined = ncomb;
  m->sky = sky;
  m->effGain = gain * texp * ncomb;
  m->rnAduSq = rn * rn / (m->effGain * m->effGain);
  return 0;
}

int imfit_AddOversampledPsfInfo(imfit_model_t m, const double *psf, int nc, int nr, int scale, int x1, int x2,
                                int y1, int y2, int normalize) {
  GET(m);
  if (!psf) return m->fail(IMFIT_E_ARG, "null PSF");
  return m->addRegion(psf, nc, nr, scale, x1, x2, y1, y2, normalize);
}

int imfit_AddErrorVector(imfit_model_t m, long n, int nc, int nr, const double *pix, int type) {
  GET(m);
  if (!pix || n != m->nDataVals || nc != m->nDataCols || nr != m->nDataRows)
    return m->fail(IMFIT_E_ARG, "error image size does not match the data");
  std::vector<double> w(pix, pix + n);
  switch (type) {  // core/model_object.cpp:595-617
    case IMFIT_WEIGHTS_ARE_SIGMAS: for (auto &v : w) v = 1.0 / v; break;
    case IMFIT_WEIGHTS_ARE_VARIANCES: for (auto &v : w) v = 1.0 / sqrt(v); break;
    case IMFIT_WEIGHTS_ARE_WEIGHTS: for (auto &v : w) v = sqrt(v); break;
    default: m->weightValsSet = false; return m->fail(IMFIT_E_ARG, "incorrect input-type specification");
  }
  m->weight = w;
  m->weightValsSet = true;
  m->externalErrors = true;
  return 0;
}

int imfit_AddMaskVector(imfit_model_t m, long n, int nc, int nr, const double *pix, int type) {
  GET(m);
  if (!pix || n != m->nDataVals || nc != m->nDataCols || nr != m->nDataRows)
    return m->fail(IMFIT_E_ARG, "mask size does not match the data");
  std::vector<double> mk(pix, pix + n);
  long valid = 0;
  if (type == IMFIT_MASK_ZERO_IS_GOOD) {
    for (auto &v : mk) {
      if (!std::isfinite(v) || v > 0.0) v = 0.0;
      else { v = 1.0; valid++; }
    }
  } else if (type == IMFIT_MASK_ZERO_IS_BAD) {
    for (auto &v : mk) {
      if (!std::isfinite(v) || v < 1.0) v = 0.0;
      else { v = 1.0; valid++; }
    }
  } else {
    m->maskExists = false;
    return m->fail(-1, "unknown mask inputType");
  }
  m->mask = mk;
  m->nValid = valid;
  m->maskExists = true;
  return 0;
}

int imfit_UseCashStatistic(imfit_model_t m) {
  GET(m);
  if (!m->dataValsSet && m->nDataVals == 0) return m->fail(IMFIT_E_STATE, "no image size yet");
  m->useCash = true;
  m->weight.assign(m->nDataVals, 1.0);
  if (m->extra.empty()) m->extra.assign(m->nDataVals, 0.0);
  m->weightValsSet = true;
  return 0;
}

int imfit_UsePoissonMLR(imfit_model_t m) {
  GET(m);
  m->pmlr = true;
  return imfit_UseCashStatistic(m);
}

int imfit_UseModelErrors(imfit_model_t m) {
  GET(m);
  m->modelErrors = true;
  m->dataErrors = false;
  m->weight.assign(m->nDataVals, 1.0);
  m->weightValsSet = true;
  return 0;
}

int imfit_FinalSetupForFitting(imfit_model_t m) {
  GET(m);
  return m->finalSetup();
}

int imfit_SetMaxThreads(imfit_model_t m, int) { GET(m); return 0; }
int imfit_SetOMPChunkSize(imfit_model_t m, int) { GET(m); return 0; }

int imfit_GetNParams(imfit_model_t m) { return m ? m->nParamsTot : IMFIT_E_ARG; }
long imfit_GetNDataValues(imfit_model_t m) { return m ? m->nDataVals : IMFIT_E_ARG; }
long imfit_GetNValidPixels(imfit_model_t m) { return m ? m->nValid : IMFIT_E_ARG; }
int imfit_GetNFunctions(imfit_model_t m) { return m ? (int)m->funcs.size() : IMFIT_E_ARG; }

int imfit_WhichFitStatistic(imfit_model_t m, int verbose) {
  if (!m) return IMFIT_E_ARG;
  if (m->useCash) return m->pmlr ? IMFIT_FITSTAT_POISSON_MLR : IMFIT_FITSTAT_CASH;
  if (!verbose) return IMFIT_FITSTAT_CHISQUARE;
  if (m->modelErrors) return IMFIT_FITSTAT_CHISQUARE_MODEL;
  if (m->externalErrors) return IMFIT_FITSTAT_CHISQUARE_USER;
  return IMFIT_FITSTAT_CHISQUARE_DATA;
}

int imfit_GetModelImageSize(imfit_model_t m, int *nc, int *nr) {
  if (!m || !nc || !nr) return IMFIT_E_ARG;
  *nc = m->nModelCols;
  *nr = m->nModelRows;
  return 0;
}

int imfit_CreateModelImage(imfit_model_t m, const double *params) {
  GET(m);
  if (!params) return m->fail(IMFIT_E_ARG, "null parameter vector");
  return m->createModelImage(params);
}

int imfit_ComputeModelImage(imfit_model_t m, const double *params) { return imfit_CreateModelImage(m, params); }

int imfit_ComputeDeviates(imfit_model_t m, double *y, const double *params) {
  GET(m);
  if (!y || !params) return m->fail(IMFIT_E_ARG, "null argument");
  return m->computeDeviates(y, params);
}

int imfit_GetFitStatistic(imfit_model_t m, const double *params, double *s) {
  GET(m);
  if (!s || !params) return m->fail(IMFIT_E_ARG, "null argument");
  return m->getFitStatistic(params, s);
}

int imfit_ChiSquared(imfit_model_t m, const double *params, double *s) {
  GET(m);
  if (!s || !params) return m->fail(IMFIT_E_ARG, "null argument");
  return m->getFitStatistic(params, s, 0);
}

int imfit_CashStatistic(imfit_model_t m, const double *params, double *s) {
  GET(m);
  if (!s || !params) return m->fail(IMFIT_E_ARG, "null argument");
  if (!m->useCash) return m->fail(IMFIT_E_STATE, "Cash statistic needs UseCashStatistic");
  return m->getFitStatistic(params, s, 1);
}

int imfit_GetModelImageVector(imfit_model_t m, double *out) {
  GET(m);
  if (!out) return IMFIT_E_ARG;
  if (!m->modelComputed) return m->fail(IMFIT_E_STATE, "Model image has not yet been computed");
  DevBuf<double> tmp;
  cudaError_t e = tmp.reserve(m->nDataVals);
  if (!e)
    e = launch_crop64(m->dModel.p, m->nModelCols, m->doConv ? m->nPsfRows : 0, m->doConv ? m->nPsfCols : 0,
                      m->nDataCols, m->nDataRows, tmp.p, m->stream);
  if (!e) e = cudaMemcpyAsync(out, tmp.p, sizeof(double) * m->nDataVals, cudaMemcpyDeviceToHost, m->stream);
  if (!e) e = cudaStreamSynchronize(m->stream);
  return e ? m->cuda_fail(e, "GetModelImageVector") : 0;
}

int imfit_GetExpandedModelImageVector(imfit_model_t m, double *out) {
  GET(m);
  if (!out) return IMFIT_E_ARG;
  if (!m->modelComputed) return m->fail(IMFIT_E_STATE, "Model image has not yet been computed");
  cudaError_t e = cudaMemcpyAsync(out, m->dModel.p, sizeof(double) * m->nModelVals, cudaMemcpyDeviceToHost, m->stream);
  if (!e) e = cudaStreamSynchronize(m->stream);
  return e ? m->cuda_fail(e, "GetExpandedModelImageVector") : 0;
}

int imfit_GetResidualImageVector(imfit_model_t m, double *out) {
  GET(m);
  int st = imfit_GetModelImageVector(m, out);
  if (st) return st;
  for (long z = 0; z < m->nDataVals; z++) out[z] = m->data[z] - out[z];
  return 0;
}

int imfit_GetWeightImageVector(imfit_model_t m, double *out) {
  GET(m);
  if (!out) return IMFIT_E_ARG;
  if (!m->weightValsSet) return m->fail(IMFIT_E_STATE, "Weight image has not yet been computed");
  std::vector<double> w = m->weight;
  if (m->modelErrors && m->finalSetupDone) {
    cudaError_t e = cudaMemcpy(w.data(), m->dWeight.p, sizeof(double) * m->nDataVals, cudaMemcpyDeviceToHost);
    if (e) return m->cuda_fail(e, "GetWeightImageVector");
  }
  for (long z = 0; z < m->nDataVals; z++) out[z] = w[z] * w[z];
  return 0;
}

int imfit_GetDataVector(imfit_model_t m, double *out) {
  GET(m);
  if (!out || !m->dataValsSet) return m->fail(IMFIT_E_STATE, "Image data values have not yet been supplied");
  memcpy(out, m->data.data(), sizeof(double) * m->nDataVals);
  return 0;
}

int imfit_UseBootstrap(imfit_model_t m, unsigned long seed) {
  GET(m);
  m->rng.seed(seed);
  m->doBootstrap = true;
  return m->makeBootstrapSample();
}

int imfit_MakeBootstrapSample(imfit_model_t m) {
  GET(m);
  if (!m->doBootstrap) return m->fail(IMFIT_E_STATE, "UseBootstrap not called");
  return m->makeBootstrapSample();
}

int imfit_GetFitStatisticAndGradientFD(imfit_model_t m, const double *params, double *s, double *g) {
  GET(m);
  if (!params || !s || !g) return m->fail(IMFIT_E_ARG, "null argument");
  return m->fdGradient(params, s, g);
}

int imfit_GetFitStatisticAndGradient(imfit_model_t m, const double *params, double *s, double *g) {
  GET(m);
  if (!params || !s || !g) return m->fail(IMFIT_E_ARG, "null argument");
  return m->fastHost(1, params, s, g);
}

int imfit_GetFitStatisticFast(imfit_model_t m, const double *params, double *s) {
  GET(m);
  if (!params || !s) return m->fail(IMFIT_E_ARG, "null argument");
  return m->fastHost(1, params, s, nullptr);
}

int imfit_BatchFitStatisticAndGradient(imfit_model_t m, int B, const double *params, double *stats, double *grads) {
  GET(m);
  if (B < 1 || !params || !stats) return m->fail(IMFIT_E_ARG, "bad batch arguments");
  return m->fastHost(B, params, stats, grads);
}

int imfit_BatchFitStatisticAndGradientDevice(imfit_model_t m, int B, const double *dP, double *dS, double *dG) {
  GET(m);
  if (B < 1 || !dP || !dS) return m->fail(IMFIT_E_ARG, "bad batch arguments");
  return m->enqueueFast(B, dP, dS, dG);
}

int imfit_GetJacobian(imfit_model_t m, const double *params, double *fjac, double *deviates) {
  GET(m);
  if (!params || !fjac) return m->fail(IMFIT_E_ARG, "null argument");
  return m->jacobianHost(params, fjac, deviates);
}

int imfit_GetJtWJ(imfit_model_t m, const double *params, double *s, double *jtj, double *jtdev) {
  GET(m);
  if (!params || !s) return m->fail(IMFIT_E_ARG, "null argument");
  return m->jtwjHost(1, params, s, jtj, jtdev);
}

int imfit_BatchJtWJDevice(imfit_model_t m, int B, const double *dP, double *dS, double *dA, double *dB) {
  GET(m);
  if (B < 1 || !dP || !dS || !dA || !dB) return m->fail(IMFIT_E_ARG, "bad batch arguments");
  return m->enqueueJtwj(B, dP, dS, dA, dB);
}

int imfit_FitLM(imfit_model_t m, double *params, const int *fixed, const double *lower, const double *upper,
                double ftol, int maxIter, double *stat, int *nIter, int *nEval, int *status) {
  GET(m);
  if (!params) return m->fail(IMFIT_E_ARG, "null argument");
  if (!(ftol > 0.0)) return m->fail(IMFIT_E_ARG, "ftol must be positive");
  LMSettings set;
  set.ftol = ftol;
  if (maxIter > 0) set.maxIter = maxIter;
  const int n = m->nParamsTot;
  LMResult res;
  JtwjEval ev = [m, n](const double *x, double *S, double *A, double *b) {
    (void)n;
    return m->jtwjHost(1, x, S, A, b);
  };
  int st = lm_minimize(n, params, fixed, lower, upper, set, ev, res);
  if (stat) *stat = res.stat;
  if (nIter) *nIter = res.nIter;
  if (nEval) *nEval = res.nEval;
  if (status) *status = res.status;
  return st < 0 ? st : 0;
}

int imfit_MinimizeNormalEquations(int n, double *params, const int *fixed, const double *lower, const double *upper,
                                  double ftol, int maxIter, imfit_normal_eq_fn eval, void *user, double *stat,
                                  int *nIter, int *nEval, int *status) {
  if (n < 1 || !params || !eval) {
    imfit::set_global_error("MinimizeNormalEquations: bad arguments");
    return IMFIT_E_ARG;
  }
  if (!(ftol > 0.0)) {
    imfit::set_global_error("MinimizeNormalEquations: ftol must be positive");
    return IMFIT_E_ARG;
  }
  LMSettings set;
  set.ftol = ftol;
  if (maxIter > 0) set.maxIter = maxIter;
  LMResult res;
  JtwjEval ev = [eval, user](const double *x, double *S, double *A, double *b) { return eval(x, S, A, b, user); };
  int st = lm_minimize(n, params, fixed, lower, upper, set, ev, res);
  if (stat) *stat = res.stat;
  if (nIter) *nIter = res.nIter;
  if (nEval) *nEval = res.nEval;
  if (status) *status = res.status;
  if (st < 0) imfit::set_global_error("MinimizeNormalEquations: the evaluator failed");
  return st < 0 ? st : 0;
}

int imfit_MinimizeNormalEquationsBatch(int B, int n, double *params, const int *fixed, const double *lower,
                                       const double *upper, double ftol, int maxIter, imfit_normal_eq_batch_fn eval,
                                       void *user, double *statistics, int *nIter, int *status) {
  if (B < 1 || n < 1 || !params || !eval) {
    imfit::set_global_error("MinimizeNormalEquationsBatch: bad arguments");
    return IMFIT_E_ARG;
  }
  if (!(ftol > 0.0)) {
    imfit::set_global_error("MinimizeNormalEquationsBatch: ftol must be positive");
    return IMFIT_E_ARG;
  }
  LMSettings set;
  set.ftol = ftol;
  if (maxIter > 0) set.maxIter = maxIter;
  std::vector<LMResult> res((size_t)B);
  JtwjBatchEval ev = [eval, user, B](const double *X, const unsigned char *active, double *S, double *A,
                                     double *b) { return eval(B, X, active, S, A, b, user); };
  const int st = lm_minimize_batch(B, n, params, fixed, lower, upper, set, ev, res.data());
  for (int i = 0; i < B; i++) {
    if (statistics) statistics[i] = res[i].stat;
    if (nIter) nIter[i] = res[i].nIter;
    if (status) status[i] = res[i].status;
  }
  if (st < 0) imfit::set_global_error("MinimizeNormalEquationsBatch: the evaluator failed");
  return st < 0 ? st : 0;
}

int imfit_BootstrapFitBatch(imfit_model_t m, int nSamples, const double *bestfit, const int *fixed,
                            const double *lower, const double *upper, double ftol, int maxIter, double *params,
                            double *statistics, int *nIter, int *status) {
  if (!m) return IMFIT_E_ARG;
  return m->bootstrapFitBatch(nSamples, bestfit, fixed, lower, upper, ftol, maxIter, params, statistics, nIter,
                              status);
}

int imfit_FitLMBatch(imfit_model_t m, int B, double *params, const int *fixed, const double *lower,
                     const double *upper, double ftol, int maxIter, double *stats, int *nIter, int *status) {
  GET(m);
  if (B < 1 || !params) return m->fail(IMFIT_E_ARG, "bad batch arguments");
  if (!(ftol > 0.0)) return m->fail(IMFIT_E_ARG, "ftol must be positive");
  return m->fitLMBatch(B, params, fixed, lower, upper, ftol, maxIter, stats, nIter, status);
}

int imfit_GetLMBatchStats(imfit_model_t m, int *rounds, long *evaluations, double *evalSeconds, double *totalSeconds) {
  if (!m) return IMFIT_E_ARG;
  if (rounds) *rounds = m->lmStats.rounds;
  if (evaluations) *evaluations = m->lmStats.evaluations;
  if (evalSeconds) *evalSeconds = m->lmStats.evalSeconds;
  if (totalSeconds) *totalSeconds = m->lmStats.totalSeconds;
  return IMFIT_OK;
}

int imfit_SetupCutouts(imfit_model_t m, int nImg, const int *cols, const int *rows, const double *pix,
                       const double *sig, const int *psfCols, const int *psfRows, const double *psfs) {
  GET(m);
  return m->setupCutouts(nImg, cols, rows, pix, sig, psfCols, psfRows, psfs);
}

int imfit_CutoutsJtWJ(imfit_model_t m, int K, const int *cutouts, const double *params, double *stats,
                      double *jtj, double *jtdev) {
  GET(m);
  return m->ragJtwjHost(K, cutouts, params, stats, jtj, jtdev);
}

int imfit_SetupImageStack(imfit_model_t m, int nImg, int nc, int nr, const double *pix, const double *sig,
                          const double *psfs, int pc, int pr) {
  GET(m);
  return m->setupStack(nImg, nc, nr, pix, sig, psfs, pc, pr);
}

int imfit_GetSingleFunctionImage(imfit_model_t m, const double *params, int fi, double *out) {
  GET(m);
  if (!params || !out) return m->fail(IMFIT_E_ARG, "null argument");
  return m->singleFunctionImage(params, fi, out);
}

int imfit_FindTotalFluxes(imfit_model_t m, const double *params, int xSize, int ySize, double *indiv,
                          double *total) {
  GET(m);
  if (!params) return m->fail(IMFIT_E_ARG, "null argument");
  return m->findTotalFluxes(params, xSize, ySize, indiv, total);
}

int imfit_Synchronize(imfit_model_t m) {
  GET(m);
  cudaError_t e = cudaStreamSynchronize(m->stream);
  return e ? m->cuda_fail(e, "synchronize") : 0;
}

int imfit_GetStream(imfit_model_t m, void **stream) {
  GET(m);
  if (!stream) return IMFIT_E_ARG;
  *stream = (void *)m->stream;
  return 0;
}

int imfit_SetUseGraphs(imfit_model_t m, int enable) {
  GET(m);
  m->useGraphs = enable != 0;
  return 0;
}

int imfit_SetKernelTiming(imfit_model_t m, int enable) {
  GET(m);
  const bool on = enable != 0;
  if (on == m->timing) return 0;
  cudaStreamSynchronize(m->stream);
  if (on) {
    for (int i = 0; i < StageTimer::kMax; i++)
      if (cudaEventCreate(&m->timer.ev[i]) != cudaSuccess) return m->fail(IMFIT_E_CUDA, "cudaEventCreate");
  } else {
    for (int i = 0; i < StageTimer::kMax; i++) cudaEventDestroy(m->timer.ev[i]);
  }
  m->timer.n = 0;
  m->timing = on;
  if (m->graph.exec) {
    cudaGraphExecDestroy(m->graph.exec);
    m->graph = Captured{};
  }
  return 0;
}

int imfit_SetKernelTimingStage(imfit_model_t m, const char *stage) {
  GET(m);
  m->timingStage = stage ? stage : "";
  if (m->graph.exec) {
    cudaGraphExecDestroy(m->graph.exec);
    m->graph = Captured{};
  }
  return 0;
}

int imfit_SetAutotune(imfit_model_t m, int enable) {
  GET(m);
  m->autotune = enable != 0;
  m->tuned.clear();
  if (m->graph.exec) {
    cudaGraphExecDestroy(m->graph.exec);
    m->graph = Captured{};
  }
  return 0;
}

int imfit_SetLaunchShape(imfit_model_t m, int rowRpb, int rowThreads, int colCpb, int colThreads) {
  GET(m);
  if (rowRpb < 0) {
    m->hasFixedTune = false;
  } else {
    if (rowRpb < 1 || rowRpb > 4 || rowThreads < 32 || rowThreads > 1024 || rowThreads % 32 || colCpb < 0 ||
        colCpb > 8 || colThreads < 0 || colThreads > 1024 || colThreads % 32)
      return m->fail(IMFIT_E_ARG, "bad launch shape");
    m->fixedTune = FastTune{rowRpb, rowThreads, colCpb, colThreads};
    m->hasFixedTune = true;
  }
  m->tuned.clear();
  if (m->graph.exec) {
    cudaGraphExecDestroy(m->graph.exec);
    m->graph = Captured{};
  }
  return 0;
}

int imfit_SetFFTPlan(imfit_model_t m, int candidate, int radixOrder) {
  GET(m);
  if (candidate < 0) {
    m->fftPinned = false;
    m->fftTuned = false;
  } else {
    if (candidate >= imfit_model_s::kFftCandidates || radixOrder < 0 || radixOrder >= kRadixVariants)
      return m->fail(IMFIT_E_ARG, "bad FFT plan");
    m->fftCand = candidate;
    m->fftVariant = radixOrder;
    m->fftPinned = true;
  }
  m->fastReady = false;
  m->tuned.clear();
  if (m->graph.exec) {
    cudaGraphExecDestroy(m->graph.exec);
    m->graph = Captured{};
  }
  return 0;
}

int imfit_GetFFTPlan(imfit_model_t m, int *Lx, int *Ly, int *radixOrder) {
  GET(m);
  if (Lx) *Lx = m->Fx.L;
  if (Ly) *Ly = m->Fy.L;
  if (radixOrder) *radixOrder = m->fftVariant;
  return 0;
}

int imfit_GetTuning(imfit_model_t m, int *fftCandidate, int *radixOrder, int *rowsPerCta, int *rowThreads,
                    int *colsPerCta, int *colThreads) {
  GET(m);
  if (fftCandidate) *fftCandidate = m->fftCand;
  if (radixOrder) *radixOrder = m->fftVariant;
  if (rowsPerCta) *rowsPerCta = m->tune.rowRpb;
  if (rowThreads) *rowThreads = m->tune.rowThreads;
  if (colsPerCta) *colsPerCta = m->tune.colCpb;
  if (colThreads) *colThreads = m->tune.colThreads;
  return 0;
}

int imfit_GetLaunchShape(imfit_model_t m, int *rowRpb, int *rowThreads, int *colCpb) {
  GET(m);
  if (rowRpb) *rowRpb = m->tune.rowRpb;
  if (rowThreads) *rowThreads = m->tune.rowThreads;
  if (colCpb) *colCpb = m->tune.colCpb;
  return 0;
}

int imfit_SetConcurrentRegions(imfit_model_t m, int enable) {
  GET(m);
  m->concurrent = enable != 0;
  if (m->graph.exec) {
    cudaGraphExecDestroy(m->graph.exec);
    m->graph = Captured{};
  }
  return 0;
}

int imfit_GetKernelTimes(imfit_model_t m, double *ms, char *names, int namesLen, int maxN) {
  GET(m);
  if (!m->timing) return m->fail(IMFIT_E_STATE, "kernel timing is not enabled");
  cudaError_t e = cudaStreamSynchronize(m->stream);
  if (e) return m->cuda_fail(e, "GetKernelTimes");
  std::string joined;
  int k = 0;
  for (int i = 1; i < m->timer.n && k < maxN; i++, k++) {
    float t = 0.f;
    e = cudaEventElapsedTime(&t, m->timer.ev[i - 1], m->timer.ev[i]);
    if (e) return m->cuda_fail(e, "cudaEventElapsedTime");
    if (ms) ms[k] = t;
    if (!joined.empty()) joined += ",";
    joined += m->timer.names[i];
  }
  if (names && namesLen > 0) snprintf(names, namesLen, "%s", joined.c_str());
  return k;
}

int imfit_HostAlloc(unsigned long bytes, void **ptr) {
  if (!ptr) return IMFIT_E_ARG;
  cudaError_t e = cudaMallocHost(ptr, bytes ? bytes : 1);
  if (e) {
    g_createError = std::string("cudaMallocHost: ") + cudaGetErrorString(e);
    return IMFIT_E_NOMEM;
  }
  return 0;
}

int imfit_HostFree(void *ptr) {
  if (ptr) cudaFreeHost(ptr);
  return 0;
}

int imfit_GetFastModelImageVector(imfit_model_t m, const double *params, double *out) {
  GET(m);
  if (!params || !out) return m->fail(IMFIT_E_ARG, "null argument");
  int st = m->prepareFast();
  if (st) return st;
  st = m->ensureFastCap(1);
  if (st) return st;
  DevBuf<float> mo;
  cudaError_t e = mo.reserve(m->nDataVals);
  if (!e) e = cudaMemcpyAsync(m->dParams.p, params, sizeof(double) * m->nParamsTot, cudaMemcpyHostToDevice, m->stream);
  if (e) return m->cuda_fail(e, "fast model");
  st = m->enqueueFast(1, m->dParams.p, m->dStat.p, nullptr, mo.p);
  if (st) return st;
  std::vector<float> h(m->nDataVals);
  e = cudaMemcpyAsync(h.data(), mo.p, sizeof(float) * m->nDataVals, cudaMemcpyDeviceToHost, m->stream);
  if (!e) e = cudaStreamSynchronize(m->stream);
  if (e) return m->cuda_fail(e, "fast model");
  for (long z = 0; z < m->nDataVals; z++) out[z] = h[z];
  return 0;
}

}  // extern "C"
