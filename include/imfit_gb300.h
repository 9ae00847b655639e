/* imfit_gb300.h -- C ABI of the GB300 model-image / fit-statistic library.
 *
 * The entry points mirror the reference's ModelObject methods one for one
 * (core/model_object.h:38-347, core/model_object.cpp) so that a thin C++
 * subclass of ModelObject, or any FFI, can route the solvers' calls here.
 * Each declaration names the reference method it replaces.
 *
 * Conventions
 *  - Every call returns an int status: 0 on success, a negative IMFIT_E_*
 *    code on failure (imfit_LastError gives the message).  Nothing aborts.
 *  - Images are row-major double arrays, x (column) fastest, row 0 first --
 *    the reference's pixel-vector layout.
 *  - Host arrays passed in are copied; nothing is borrowed after the call
 *    returns (the reference borrows data/mask/error arrays and rewrites them
 *    in place; here the converted weights/mask can be read back with the
 *    Get* calls).
 *  - One handle is used by one host thread at a time, like a ModelObject.
 */
#ifndef IMFIT_GB300_H
#define IMFIT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct imfit_model_s *imfit_model_t;

#define IMFIT_OK 0
#define IMFIT_E_ARG (-1)        /* invalid argument or call order */
#define IMFIT_E_CUDA (-2)       /* CUDA runtime error */
#define IMFIT_E_NOMEM (-3)      /* device allocation failed */
#define IMFIT_E_UNSUPPORTED (-4) /* valid for the reference, not supported on this path */
#define IMFIT_E_STATE (-5)      /* required setup step missing */

/* error-weight and mask input types (core/definitions.h) */
#define IMFIT_WEIGHTS_ARE_SIGMAS 100
#define IMFIT_WEIGHTS_ARE_VARIANCES 110
#define IMFIT_WEIGHTS_ARE_WEIGHTS 120
#define IMFIT_MASK_ZERO_IS_GOOD 10
#define IMFIT_MASK_ZERO_IS_BAD 20

/* fit-statistic codes (core/definitions.h) */
#define IMFIT_FITSTAT_CHISQUARE 1
#define IMFIT_FITSTAT_CASH 2
#define IMFIT_FITSTAT_POISSON_MLR 3
#define IMFIT_FITSTAT_CHISQUARE_DATA 10
#define IMFIT_FITSTAT_CHISQUARE_MODEL 11
#define IMFIT_FITSTAT_CHISQUARE_USER 12

/* ---- lifetime ------------------------------------------------------------- */
/* ModelObject::ModelObject (core/model_object.cpp:108); device = CUDA ordinal */
int imfit_ModelObject_new(int device, imfit_model_t *out);
/* ModelObject::~ModelObject (core/model_object.cpp:181) */
int imfit_ModelObject_delete(imfit_model_t m);
/* message of the last failing call on this handle (or the last creation error) */
const char *imfit_LastError(imfit_model_t m);
/* version string of the library */
const char *imfit_Version(void);

/* ---- functions (FunctionObject plug-ins, by config-file name) --------------- */
/* ModelObject::AddFunction (core/model_object.cpp:279) with the factory of
 * core/add_functions.cpp:389-461: name is the config-file FUNCTION name
 * ("Sersic", "Exponential", "FlatSky", "GaussianRing", "Moffat", "Gaussian",
 * "ExponentialDisk3D", "FerrersBar3D", "PointSource", "PointSourceRot",
 * "TiltedSkyPlane"). */
int imfit_AddFunction(imfit_model_t m, const char *name);
/* FunctionObject::SetExtraParams (an OPTIONAL_PARAMS entry of the
 * configuration file) for function i: PointSource / PointSourceRot accept
 * "method" = bicubic | lanczos2 | lanczos3 (PointSourceRot: not lanczos3)
 * (function_objects/func_pointsource.cpp:140-180); every other function
 * takes none (IMFIT_E_UNSUPPORTED, as SetExtraParams returns -1). */
int imfit_SetFunctionOptionalParam(imfit_model_t m, int i, const char *name, const char *value);
/* FunctionObject::SetSubsampling (function_objects/function_object.cpp:78) */
int imfit_SetSubsampling(imfit_model_t m, int functionIndex, int subsample);
/* ModelObject::DefineFunctionSets (core/model_object.cpp:387) */
int imfit_DefineFunctionSets(imfit_model_t m, const int *startIndices, int nSets);
/* ModelObject::PopulateParameterNames (core/model_object.cpp:2169) */
int imfit_PopulateParameterNames(imfit_model_t m);
/* ModelObject::GetParameterName (core/model_object.cpp:2186); copies into buf */
int imfit_GetParameterName(imfit_model_t m, int i, char *buf, int bufLen);

/* ---- image setup ------------------------------------------------------------ */
/* ModelObject::AddPSFVector (core/model_object.cpp:827); must precede SetupModelImage */
int imfit_AddPSFVector(imfit_model_t m, long nPixels, int nColumns, int nRows, const double *psf,
                       int normalize);
/* ModelObject::SetupModelImage (core/model_object.cpp:488) */
int imfit_SetupModelImage(imfit_model_t m, int nColumns, int nRows);
/* ModelObject::AddImageDataVector (core/model_object.cpp:462) */
int imfit_AddImageDataVector(imfit_model_t m, const double *pixels, int nColumns, int nRows);
/* ModelObject::AddImageCharacteristics (core/model_object.cpp:532) */
int imfit_AddImageCharacteristics(imfit_model_t m, double gain, double readNoise, double expTime,
                                  int nCombined, double originalSky);
/* ModelObject::AddOversampledPsfInfo (core/model_object.cpp:881), with the
 * PsfOversamplingInfo fields flattened: region x1:x2,y1:y2 in 1-based pixels */
int imfit_AddOversampledPsfInfo(imfit_model_t m, const double *psf, int nColumns, int nRows,
                                int scale, int x1, int x2, int y1, int y2, int normalize);
/* ModelObject::AddErrorVector (core/model_object.cpp:573) */
int imfit_AddErrorVector(imfit_model_t m, long nDataValues, int nColumns, int nRows,
                         const double *pixels, int inputType);
/* ModelObject::AddMaskVector (core/model_object.cpp:721) */
int imfit_AddMaskVector(imfit_model_t m, long nDataValues, int nColumns, int nRows,
                        const double *pixels, int inputType);
/* ModelObject::UseCashStatistic (core/model_object.cpp:1541) */
int imfit_UseCashStatistic(imfit_model_t m);
/* ModelObject::UsePoissonMLR (core/model_object.cpp:1583) */
int imfit_UsePoissonMLR(imfit_model_t m);
/* ModelObject::UseModelErrors (core/model_object.cpp:1501) */
int imfit_UseModelErrors(imfit_model_t m);
/* ModelObject::FinalSetupForFitting (core/model_object.cpp:967); returns 0, -1, -2, -3 */
int imfit_FinalSetupForFitting(imfit_model_t m);
/* ModelObject::SetMaxThreads / SetOMPChunkSize (core/model_object.cpp:248, 260):
 * accepted and ignored (the GPU decides its own parallelism) */
int imfit_SetMaxThreads(imfit_model_t m, int n);
int imfit_SetOMPChunkSize(imfit_model_t m, int n);

/* ---- queries ---------------------------------------------------------------- */
int imfit_GetNParams(imfit_model_t m);           /* core/model_object.cpp:2207 */
long imfit_GetNDataValues(imfit_model_t m);      /* core/model_object.cpp:2215 */
long imfit_GetNValidPixels(imfit_model_t m);     /* core/model_object.cpp:2223 */
int imfit_GetNFunctions(imfit_model_t m);        /* core/model_object.cpp:2199 */
int imfit_WhichFitStatistic(imfit_model_t m, int verbose); /* core/model_object.cpp:1592 */
/* size of the expanded (PSF-padded) model image of GetExpandedModelImageVector */
int imfit_GetModelImageSize(imfit_model_t m, int *nColumns, int *nRows);

/* ---- the plain FP64 path (drop-in) ------------------------------------------ */
/* ModelObject::CreateModelImage (core/model_object.cpp:1103) */
int imfit_CreateModelImage(imfit_model_t m, const double *params);
/* alias of imfit_CreateModelImage under the name used in some documentation */
int imfit_ComputeModelImage(imfit_model_t m, const double *params);
/* ModelObject::ComputeDeviates (core/model_object.cpp:1413); yResults holds
 * GetNDataValues() doubles, or GetNValidPixels() in bootstrap mode */
int imfit_ComputeDeviates(imfit_model_t m, double *yResults, const double *params);
/* ModelObject::GetFitStatistic (core/model_object.cpp:1620) */
int imfit_GetFitStatistic(imfit_model_t m, const double *params, double *statistic);
/* ModelObject::ChiSquared (core/model_object.cpp:1633) */
int imfit_ChiSquared(imfit_model_t m, const double *params, double *statistic);
/* ModelObject::CashStatistic (core/model_object.cpp:1703) */
int imfit_CashStatistic(imfit_model_t m, const double *params, double *statistic);
/* ModelObject::GetModelImageVector (core/model_object.cpp:2257): data-sized crop */
int imfit_GetModelImageVector(imfit_model_t m, double *out);
/* ModelObject::GetExpandedModelImageVector (core/model_object.cpp:2296) */
int imfit_GetExpandedModelImageVector(imfit_model_t m, double *out);
/* ModelObject::GetResidualImageVector (core/model_object.cpp:2312) */
int imfit_GetResidualImageVector(imfit_model_t m, double *out);
/* ModelObject::GetWeightImageVector (core/model_object.cpp:2359): 1/sigma^2 */
int imfit_GetWeightImageVector(imfit_model_t m, double *out);
/* ModelObject::GetSingleFunctionImage (core/model_object.cpp:1241): the image
 * of function functionIndex alone (convolved, oversampled regions included),
 * data-sized; like the reference it replaces the stored model image. */
int imfit_GetSingleFunctionImage(imfit_model_t m, const double *params, int functionIndex, double *out);
/* ModelObject::FindTotalFluxes (core/model_object.cpp:2415): each function
 * centred on an xSize x ySize image, its analytic TotalFlux where the class
 * has one, otherwise the sum of its values over that image (FP64, GPU);
 * individualFluxes (GetNFunctions() values) and totalFlux may be NULL. */
int imfit_FindTotalFluxes(imfit_model_t m, const double *params, int xSize, int ySize, double *individualFluxes,
                          double *totalFlux);
/* ModelObject::GetDataVector (core/model_object.cpp:2383) */
int imfit_GetDataVector(imfit_model_t m, double *out);
/* ModelObject::UseBootstrap (core/model_object.cpp:2042), seeding MT19937 like
 * core/bootstrap_errors.cpp:176 */
int imfit_UseBootstrap(imfit_model_t m, unsigned long seed);
/* ModelObject::MakeBootstrapSample (core/model_object.cpp:2061) */
int imfit_MakeBootstrapSample(imfit_model_t m);

/* ---- gradients (no counterpart in the reference) ---------------------------- */
/* Statistic and its gradient w.r.t. all GetNParams() parameters by the plain
 * FP64 model and a one-sided finite difference per parameter, with mpfit's
 * step rule h = sqrt(eps)*|x| (solvers/mpfit.cpp:1194, 1254-1258):
 * 1 + nParams model evaluations.  For chi^2 the gradient is 2 J^T dev with J
 * the forward-difference Jacobian of the deviates, as mpfit forms it. */
int imfit_GetFitStatisticAndGradientFD(imfit_model_t m, const double *params, double *statistic,
                                       double *gradient);
/* Statistic and gradient by the fast path: FP32 model evaluation and FFTs,
 * FP64 geometry setup and reductions, adjoint (reverse-mode) gradient. */
int imfit_GetFitStatisticAndGradient(imfit_model_t m, const double *params, double *statistic,
                                     double *gradient);
/* Fast-path statistic only (FP32 evaluation, FP64 reduction) */
int imfit_GetFitStatisticFast(imfit_model_t m, const double *params, double *statistic);
/* Batched fast path over nBatch parameter vectors (params: nBatch x nParams,
 * row-major).  Host buffers; gradients may be NULL for statistics only. */
int imfit_BatchFitStatisticAndGradient(imfit_model_t m, int nBatch, const double *params,
                                       double *statistics, double *gradients);
/* Same with DEVICE pointers on the handle's stream (no host copies); the
 * call returns once the work is enqueued.  imfit_Synchronize waits. */
int imfit_BatchFitStatisticAndGradientDevice(imfit_model_t m, int nBatch, const double *d_params,
                                             double *d_statistics, double *d_gradients);
/* Gauss-Newton normal equations of the deviates by the fast path, forward
 * mode: the PSF-convolved derivative image of every parameter (one batched
 * FFT convolution), then jtj = J^T J (nParams x nParams, row-major),
 * jtdev = J^T dev and statistic = sum dev^2, with J = d dev / d params the
 * analytic Jacobian mpfit approximates by finite differences
 * (solvers/mpfit.cpp:1102-1356).  The gradient of the statistic is 2 jtdev.
 * chi^2 (data, external or model-based errors) and Poisson-MLR; the Cash
 * statistic has no deviates and returns IMFIT_E_UNSUPPORTED. */
int imfit_GetJtWJ(imfit_model_t m, const double *params, double *statistic, double *jtj, double *jtdev);
/* Analytic Jacobian of the deviates by the same forward-mode pass: fjac is
 * column-major, GetNDataValues() values per parameter, column j = d dev /
 * d param_j in ComputeDeviates' order -- the derivative vectors mpfit takes
 * from a user function for parameters with side = 3 (solvers/mpfit.cpp:1210-1232),
 * replacing its finite differences.  deviates (may be NULL) receives the
 * deviates at params (FP32-evaluated).  chi^2 and Poisson-MLR; not with a
 * bootstrap sample, an image stack or 3-D components. */
int imfit_GetJacobian(imfit_model_t m, const double *params, double *fjac, double *deviates);
/* Batched form on DEVICE pointers (nBatch x nParams in, nBatch, nBatch x
 * nParams^2 and nBatch x nParams out), enqueued on the handle's stream. */
int imfit_BatchJtWJDevice(imfit_model_t m, int nBatch, const double *d_params, double *d_statistics,
                          double *d_jtj, double *d_jtdev);
/* Levenberg-Marquardt fit (FP64 normal-equation solve on the host, JtWJ from
 * imfit_GetJtWJ): mpfit's trust-region iteration (solvers/mpfit.cpp:551-1060:
 * column-norm scaling, lmpar damping, whole-step scaling at limits, its ftol
 * and xtol tests).  params: start values in, fitted values out.  fixed (may be
 * NULL): nonzero = held fixed.  lower/upper (may be NULL): limits, used where
 * lower < upper.  ftol: relative-reduction tolerance (the reference's default
 * is 1e-8, core/definitions.h:61); maxIter <= 0 selects 1000
 * (solvers/levmar_fit.cpp:38).  Outputs (each may be NULL): the fast-path
 * statistic at the result, iterations, JtWJ evaluations, and a status
 * (1 ftol, 2 xtol: trust radius below 1e-10 of the scaled parameter norm,
 * 3 no step can be formed, 4 stalled: no progress above the FP32 noise of
 * the statistic for 20 rounds, 5 iteration limit).  Returns 0 or a
 * negative IMFIT_E_* code. */
int imfit_FitLM(imfit_model_t m, double *params, const int *fixed, const double *lower, const double *upper,
                double ftol, int maxIter, double *statistic, int *nIter, int *nEval, int *status);
/* Levenberg-Marquardt on nBatch problems at once (lockstep: one batched JtWJ
 * evaluation per round for all of them; each problem keeps its own damping
 * and convergence state).  params: nBatch x nParams in/out; fixed: nParams
 * flags shared by all (may be NULL); lower/upper: nBatch x nParams or NULL.
 * On an image stack (imfit_SetupImageStack) problem b fits image b and
 * nBatch must equal the stack size; otherwise all problems fit this
 * handle's image (e.g. several starting points).  statistics, nIter, status
 * (nBatch each) may be NULL; status codes as imfit_FitLM. */
int imfit_FitLMBatch(imfit_model_t m, int nBatch, double *params, const int *fixed, const double *lower,
                     const double *upper, double ftol, int maxIter, double *statistics, int *nIter, int *status);
/* Timing of the most recent imfit_FitLMBatch: the J^T W J evaluations (rounds
 * of the lockstep LM, problem evaluations over them, wall seconds inside
 * them, device work and transfers included) and the call's total wall
 * seconds (the rest is the host's LM steps).  Any pointer may be NULL. */
int imfit_GetLMBatchStats(imfit_model_t m, int *rounds, long *evaluations, double *evalSeconds, double *totalSeconds);
/* The Levenberg-Marquardt driver of imfit_FitLM on normal equations the
 * caller supplies: eval(x, &S, A, b, user) fills the statistic S, A = J^T J
 * (n x n, row-major) and b = J^T dev of its deviates at x and returns 0 (or a
 * negative code, which stops the fit).  For models assembled on the host from
 * several handles -- multimfit's ModelObjectMultImage
 * (core/model_object_multimage.cpp:319-441): S = sum S_i, A = sum T_i^T A_i T_i,
 * b = sum T_i^T b_i with T_i the Jacobian of image i's parameter vector.
 * Errors: imfit_LastError(NULL). */
typedef int (*imfit_normal_eq_fn)(const double *x, double *statistic, double *A, double *b, void *user);
int imfit_MinimizeNormalEquations(int n, double *params, const int *fixed, const double *lower, const double *upper,
                                  double ftol, int maxIter, imfit_normal_eq_fn eval, void *user, double *statistic,
                                  int *nIter, int *nEval, int *status);
/* The same driver over B independent problems of n parameters, stepped in
 * lockstep (the form imfit_FitLMBatch uses for cutout batches): each round
 * calls eval(B, X, active, S, A, b, user) once for the trial vectors X (B x n)
 * of the problems still running (active[i] = 1; the others' rows must be left
 * untouched), which fills S[i], A (B x n x n) and b (B x n).  params (B x n)
 * holds the starts and receives the results; fixed (n) is shared, lower and
 * upper (B x n) are per problem or NULL; statistics, nIter and status (B) may
 * be NULL.  The host steps of a large batch run on a pool of worker threads.
 * No counterpart in the reference (its fits are one at a time:
 * core/bootstrap_errors.cpp:205-215, core/model_object_multimage.cpp:353,437).
 * Errors: imfit_LastError(NULL). */
typedef int (*imfit_normal_eq_batch_fn)(int B, const double *X, const unsigned char *active, double *statistics,
                                        double *A, double *b, void *user);
int imfit_MinimizeNormalEquationsBatch(int B, int n, double *params, const int *fixed, const double *lower,
                                       const double *upper, double ftol, int maxIter, imfit_normal_eq_batch_fn eval,
                                       void *user, double *statistics, int *nIter, int *status);
/* Bootstrap refits, replacing the loop of BootstrapErrorsBase
 * (core/bootstrap_errors.cpp:160-240: MakeBootstrapSample, then LevMarFit from
 * the best-fit vector, per iteration): draws the next nSamples samples of the
 * MT19937 stream seeded by imfit_UseBootstrap (the same index sequence as the
 * reference's iterations), holds each as per-pixel multiplicities and fits all
 * of them at once with the batched LM from bestfit.  fixed, lower, upper:
 * nParams each (shared; NULL allowed).  params: nSamples x nParams out;
 * statistics, nIter, status: nSamples each (may be NULL), status codes as
 * imfit_FitLM (> 0: success).  chi^2 or Poisson-MLR. */
int imfit_BootstrapFitBatch(imfit_model_t m, int nSamples, const double *bestfit, const int *fixed,
                            const double *lower, const double *upper, double ftol, int maxIter, double *params,
                            double *statistics, int *nIter, int *status);

/* ---- image stacks (fast path; no counterpart in the reference) ------------- */
/* Many cutouts fitted with one model: nImages images of nColumns x nRows
 * pixels (row-major, image after image), per-pixel sigmas (internal weight
 * 1/sigma as AddErrorVector with WEIGHTS_ARE_SIGMAS; sigma <= 0 or
 * non-finite, or non-finite data, masks a pixel -- pad smaller cutouts this
 * way) and one psfColumns x psfRows PSF per image (normalised as the
 * reference's Convolver does).  Replaces AddImageDataVector ..
 * FinalSetupForFitting for this handle; chi^2 statistic; fast-path entry
 * points then take exactly nImages parameter vectors, vector b for image b.
 * The plain FP64 entry points are per image and reject a stack. */
int imfit_SetupImageStack(imfit_model_t m, int nImages, int nColumns, int nRows, const double *pixels,
                          const double *sigmas, const double *psfs, int psfColumns, int psfRows);
/* ---- cutout sets (fast path; no counterpart in the reference, which fits
 * its images one after another, core/bootstrap_errors.cpp:205-215) ---------- */
/* Many cutouts of DIFFERENT sizes fitted with one model in one handle, each
 * at its own size with its own PSF and FFT plan (no padding to a common
 * size).  Cutout i has columns[i] x rows[i] pixels; pixels and sigmas hold
 * the cutouts one after another (row-major each); psfColumns[i] x psfRows[i]
 * (odd) PSFs likewise in psfs, normalised as the reference's Convolver does.
 * sigma <= 0 or non-finite, or non-finite data, masks a pixel.  chi^2 only;
 * pixel functions only (no 3-D functions, point sources or oversampled
 * regions).  Every stage of an evaluation is one kernel launch over all the
 * cutouts being evaluated.  imfit_FitLMBatch then fits nImages vectors,
 * vector i to cutout i (the active cutouts of each round in one launch per
 * stage). */
int imfit_SetupCutouts(imfit_model_t m, int nImages, const int *columns, const int *rows, const double *pixels,
                       const double *sigmas, const int *psfColumns, const int *psfRows, const double *psfs);
/* Statistic, J^T J (nParams x nParams) and J^T dev of the cutouts
 * cutouts[0..K) at params (K x nParams), on the host; outputs K, K x nParams^2
 * and K x nParams values in the same order. */
int imfit_CutoutsJtWJ(imfit_model_t m, int K, const int *cutouts, const double *params, double *statistics,
                      double *jtj, double *jtdev);
int imfit_Synchronize(imfit_model_t m);
/* The CUDA stream (cudaStream_t) all work of this handle is enqueued on. */
int imfit_GetStream(imfit_model_t m, void **stream);
/* Record the fast batched evaluation for nBatch vectors as a CUDA graph and
 * replay it on later calls with the same nBatch and device pointers. */
int imfit_SetUseGraphs(imfit_model_t m, int enable);
/* FP32 model image of the fast path (data-sized), for diagnostics */
int imfit_GetFastModelImageVector(imfit_model_t m, const double *params, double *out);
/* Per-kernel timing of the fast path with CUDA events recorded on the
 * handle's stream after every kernel (also inside captured graphs).
 * GetKernelTimes synchronizes, writes the elapsed milliseconds of each kernel
 * of the most recent fast evaluation and their comma-separated names, and
 * returns the number of kernels. */
int imfit_SetKernelTiming(imfit_model_t m, int enable);
int imfit_GetKernelTimes(imfit_model_t m, double *ms, char *names, int namesLen, int maxN);
/* Restrict the timing to one named stage (two events around that kernel
 * only), or pass NULL to time every stage (then the stages run serially). */
int imfit_SetKernelTimingStage(imfit_model_t m, const char *stage);
/* Run the oversampled-region pipeline on a second stream concurrently with
 * the main-window pipeline (default on). */
int imfit_SetConcurrentRegions(imfit_model_t m, int enable);
/* Autotuning of the fast path (default on): the first fast call for each
 * batch size times FFT plans (padded lengths x radix orders; again for a batch
 * four times larger) and row/column CTA shapes on that call's parameters --
 * graph replays of the statistic + gradient evaluation, each from an empty
 * L2 -- and keeps the fastest; statistic-only calls use the same choice.
 * GetLaunchShape and GetFFTPlan report it. */
int imfit_SetAutotune(imfit_model_t m, int enable);
int imfit_GetLaunchShape(imfit_model_t m, int *rowsPerCta, int *rowThreads, int *colsPerCta);
/* Pin the fast path's launch shape instead of autotuning (rowsPerCta < 0
 * returns to autotuning): rows per CTA 1..4 and threads per row CTA; columns
 * per CTA 1..8 of the column FFT (0: automatic) and threads per column CTA
 * (0: automatic). */
int imfit_SetLaunchShape(imfit_model_t m, int rowsPerCta, int rowThreads, int colsPerCta, int colThreads);
/* Measured MUFU (SFU) throughput of a device, in transcendental operations per
 * second (lg2.approx / ex2.approx, every SM at full occupancy, CUDA events,
 * best of three): the P_SFU of the per-unit roofline
 * T_roof = bytes / HBM bandwidth + SFU operations / P_SFU.  Measurement helper
 * with no counterpart in the reference; it changes no device setting. */
int imfit_MeasureSfuRate(int device, double *opsPerSecond);
/* FFT plan of the fast path (no counterpart in the reference, which plans
 * FFTW with FFTW_ESTIMATE on the smallest padded size, core/convolver.cpp:253-256).
 * The padded length of each axis is one of the three smallest 7-smooth even
 * lengths >= the window (within 10 %), the radix order one of three
 * (0: radix 8, 9, 4, 2 then 3, 5, 7; 1: 7, 5, 9, 3 then 8, 4, 2; 2: 4, 2, 9
 * then 3, 5, 7).  By default the autotuner times every pair on the first fast call
 * and keeps the fastest; SetFFTPlan pins candidate (0..2) and order (0..2), or
 * returns to autotuning with candidate < 0.  GetFFTPlan reports the lengths
 * in use (Lx, Ly of the main window) and the order. */
int imfit_SetFFTPlan(imfit_model_t m, int candidate, int radixOrder);
int imfit_GetFFTPlan(imfit_model_t m, int *Lx, int *Ly, int *radixOrder);
/* Everything the tuning chose, in the arguments SetFFTPlan and SetLaunchShape
 * take (so that a run can be repeated with the same plan and shape, e.g.
 * under a profiler): padded-length candidate, radix order, rows per row CTA,
 * threads per row CTA, columns per column CTA, threads per column CTA (0:
 * automatic).  Any pointer may be NULL. */
int imfit_GetTuning(imfit_model_t m, int *fftCandidate, int *radixOrder, int *rowsPerCta, int *rowThreads,
                    int *colsPerCta, int *colThreads);
/* Page-locked host memory for the host-buffer entry points (cudaMallocHost). */
int imfit_HostAlloc(unsigned long bytes, void **ptr);
int imfit_HostFree(void *ptr);

/* ---- allocation-free statistic (no counterpart in the reference) ----------- */
/* chi^2 = sum over pixels of (weight * (data - model))^2, summed with the
 * same MINPACK-enorm reduction as imfit_ChiSquared, for callers that must not
 * allocate device memory when they ask for it: plug-ins of host frameworks
 * that reserve all device memory up front, deployments with a fixed device
 * budget, and solver loops that cannot afford the allocator's locking or the
 * synchronisation cudaFree implies.
 *   d_model, d_data, d_weight : nPixels device doubles each (the model already
 *                               cropped to the data; weights are 1/sigma, 0 where masked)
 *   d_result                  : one device double receiving chi^2
 *   stream                    : cudaStream_t to run on (NULL = legacy default stream)
 * Nothing is allocated: the per-block partial sums live in one fixed
 * file-scope device array of IMFIT_NOALLOC_MAX_BLOCKS * 5 doubles (160 KiB)
 * that every GPU using the library keeps until the process exits.  Inputs
 * larger than IMFIT_NOALLOC_MAX_PIXELS are rejected with IMFIT_E_ARG (see
 * imfit_LastError(NULL)).  The first call in each CUDA context looks up the
 * array's device address (with that context's device current) and caches it
 * under the context's driver ID, so a context re-created after
 * cudaDeviceReset looks it up afresh; make that first call before any stream
 * capture.  All calls share the one array, so calls that overlap on
 * the GPU (different streams, or different host threads, on one device)
 * race; serialise them.  The call only enqueues work on `stream`. */
#define IMFIT_NOALLOC_MAX_BLOCKS 4096
#define IMFIT_NOALLOC_MAX_PIXELS (IMFIT_NOALLOC_MAX_BLOCKS * 2048L)
int imfit_ChiSquaredDeviceNoAlloc(const double *d_model, const double *d_data, const double *d_weight,
                                  long nPixels, double *d_result, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* IMFIT_GB300_H */
