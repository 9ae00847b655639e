// ref_capi.cpp -- extern "C" driver for the REFERENCE's own ModelObject,
// compiled together with the reference's unmodified hot-path sources into
// oracle/_ref/libimfit_ref.so by oracle/Makefile.
//
// TEST INFRASTRUCTURE ONLY: used to pin the C restatement (imfit_oracle.c)
// and to produce golden fixtures; nothing in the product links it.
//
// The call order mirrors the reference's SetupModelObject
// (core/setup_model_object.cpp:36-157) and AddFunctions
// (core/add_functions.cpp:389-461), restricted to the function classes on the
// hot path.  The reference borrows the data/mask/error arrays and mutates
// them in place (core/model_object.cpp:468, 587, 731), so this wrapper keeps
// private copies alive for the lifetime of the model.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "model_object.h"
#include "psf_oversampling_info.h"
#include "function_objects/function_object.h"
#include "function_objects/func_sersic.h"
#include "function_objects/func_exp.h"
#include "function_objects/func_flatsky.h"
#include "function_objects/func_gaussian-ring.h"
#include "function_objects/func_moffat.h"
#include "function_objects/func_gaussian.h"
#include "function_objects/func_expdisk3d.h"
#include "function_objects/func_ferrersbar3d.h"
#include "function_objects/func_tilted-sky-plane.h"
#include "mpfit.h"
#include "mersenne_twister.h"

volatile sig_atomic_t stopSignal_flag = 0;

namespace {

FunctionObject *make_function(const char *name) {
  std::string n(name);
  if (n == "Sersic") return new Sersic();
  if (n == "Exponential") return new Exponential();
  if (n == "FlatSky") return new FlatSky();
  if (n == "GaussianRing") return new GaussianRing();
  if (n == "Moffat") return new Moffat();
  if (n == "Gaussian") return new Gaussian();
  if (n == "ExponentialDisk3D") return new ExponentialDisk3D();
  if (n == "FerrersBar3D") return new FerrersBar3D();
  if (n == "TiltedSkyPlane") return new TiltedSkyPlane();
  return nullptr;
}

struct RefModel {
  ModelObject *mo = nullptr;
  std::vector<int> setStarts;
  std::vector<double> data, mask, errors, psf;
  std::vector<PsfOversamplingInfo *> osInfos;
  int nFunctions = 0;
  ~RefModel() {
    delete mo;
    for (auto *p : osInfos) delete p;
  }
};

int fdjac_func(int m, int n, double *x, double *fvec, double **dvec, ModelObject *mo) {
  (void)m; (void)n; (void)dvec;
  mo->ComputeDeviates(fvec, x);
  return 0;
}

}  // namespace

extern "C" {

void *ref_create(void) {
  RefModel *r = new RefModel();
  r->mo = new ModelObject();
  r->mo->SetVerboseLevel(-1);
  return r;
}

void ref_destroy(void *h) { delete static_cast<RefModel *>(h); }

void ref_set_max_threads(void *h, int n) { static_cast<RefModel *>(h)->mo->SetMaxThreads(n); }

int ref_add_function(void *h, const char *name, int newSet, int subsampling) {
  RefModel *r = static_cast<RefModel *>(h);
  FunctionObject *f = make_function(name);
  if (!f) return -1;
  f->SetSubsampling(subsampling != 0);
  if (newSet || r->nFunctions == 0) r->setStarts.push_back(r->nFunctions);
  r->mo->AddFunction(f);
  r->nFunctions++;
  return 0;
}

int ref_finish_functions(void *h) {
  RefModel *r = static_cast<RefModel *>(h);
  r->mo->DefineFunctionSets(r->setStarts);
  r->mo->PopulateParameterNames();
  // (FinalModelSetup is multimfit-only: imfit never calls it, and it reads
  // ModelObject::nGlobalFunctions, which the constructor leaves unset)
  return 0;
}

int ref_add_psf(void *h, int ncols, int nrows, const double *psf, int normalize) {
  RefModel *r = static_cast<RefModel *>(h);
  r->psf.assign(psf, psf + (size_t)ncols * nrows);
  return r->mo->AddPSFVector((long)ncols * nrows, ncols, nrows, r->psf.data(), normalize != 0);
}

int ref_add_oversampled_psf(void *h, int ncols, int nrows, const double *psf, int scale,
                            const char *region, int normalize) {
  RefModel *r = static_cast<RefModel *>(h);
  double *pix = (double *)fftw_malloc(sizeof(double) * (size_t)ncols * nrows);
  memcpy(pix, psf, sizeof(double) * (size_t)ncols * nrows);
  PsfOversamplingInfo *info =
      new PsfOversamplingInfo(pix, ncols, nrows, scale, std::string(region), 0, 0, true, normalize != 0);
  r->osInfos.push_back(info);
  return r->mo->AddOversampledPsfInfo(info);
}

int ref_setup_model_image(void *h, int ncols, int nrows) {
  return static_cast<RefModel *>(h)->mo->SetupModelImage(ncols, nrows);
}

int ref_add_image_data(void *h, const double *pix, int ncols, int nrows) {
  RefModel *r = static_cast<RefModel *>(h);
  r->data.assign(pix, pix + (size_t)ncols * nrows);
  return r->mo->AddImageDataVector(r->data.data(), ncols, nrows);
}

void ref_add_image_characteristics(void *h, double gain, double rn, double texp, int ncomb,
                                   double sky) {
  static_cast<RefModel *>(h)->mo->AddImageCharacteristics(gain, rn, texp, ncomb, sky);
}

int ref_add_error_vector(void *h, const double *pix, int ncols, int nrows, int type) {
  RefModel *r = static_cast<RefModel *>(h);
  r->errors.assign(pix, pix + (size_t)ncols * nrows);
  r->mo->AddErrorVector((long)ncols * nrows, ncols, nrows, r->errors.data(), type);
  return 0;
}

int ref_add_mask_vector(void *h, const double *pix, int ncols, int nrows, int type) {
  RefModel *r = static_cast<RefModel *>(h);
  r->mask.assign(pix, pix + (size_t)ncols * nrows);
  return r->mo->AddMaskVector((long)ncols * nrows, ncols, nrows, r->mask.data(), type);
}

int ref_use_cash(void *h) { return static_cast<RefModel *>(h)->mo->UseCashStatistic(); }
void ref_use_pmlr(void *h) { static_cast<RefModel *>(h)->mo->UsePoissonMLR(); }
int ref_use_model_errors(void *h) { return static_cast<RefModel *>(h)->mo->UseModelErrors(); }
int ref_final_setup(void *h) { return static_cast<RefModel *>(h)->mo->FinalSetupForFitting(); }

int ref_n_params(void *h) { return static_cast<RefModel *>(h)->mo->GetNParams(); }
long ref_n_data(void *h) { return static_cast<RefModel *>(h)->mo->GetNDataValues(); }
long ref_n_valid(void *h) { return static_cast<RefModel *>(h)->mo->GetNValidPixels(); }
int ref_which_statistic(void *h) { return static_cast<RefModel *>(h)->mo->WhichFitStatistic(true); }

void ref_create_model_image(void *h, const double *params) {
  RefModel *r = static_cast<RefModel *>(h);
  std::vector<double> p(params, params + r->mo->GetNParams());
  r->mo->CreateModelImage(p.data());
}

int ref_get_model_image(void *h, double *out) {
  RefModel *r = static_cast<RefModel *>(h);
  double *m = r->mo->GetModelImageVector();
  if (!m) return -1;
  memcpy(out, m, sizeof(double) * (size_t)r->mo->GetNDataValues());
  return 0;
}

int ref_get_expanded_model_image(void *h, double *out, long n) {
  RefModel *r = static_cast<RefModel *>(h);
  double *m = r->mo->GetExpandedModelImageVector();
  if (!m) return -1;
  memcpy(out, m, sizeof(double) * (size_t)n);
  return 0;
}

void ref_compute_deviates(void *h, double *out, const double *params) {
  RefModel *r = static_cast<RefModel *>(h);
  std::vector<double> p(params, params + r->mo->GetNParams());
  r->mo->ComputeDeviates(out, p.data());
}

double ref_get_fit_statistic(void *h, const double *params) {
  RefModel *r = static_cast<RefModel *>(h);
  std::vector<double> p(params, params + r->mo->GetNParams());
  return r->mo->GetFitStatistic(p.data());
}

int ref_get_weights(void *h, double *out) {
  RefModel *r = static_cast<RefModel *>(h);
  double *w = r->mo->GetWeightImageVector();  // 1/sigma^2 form
  if (!w) return -1;
  memcpy(out, w, sizeof(double) * (size_t)r->mo->GetNDataValues());
  return 0;
}

int ref_get_mask(void *h, double *out) {
  RefModel *r = static_cast<RefModel *>(h);
  if (r->mask.empty()) return -1;
  memcpy(out, r->mask.data(), sizeof(double) * r->mask.size());
  return 0;
}

int ref_get_data(void *h, double *out) {
  RefModel *r = static_cast<RefModel *>(h);
  memcpy(out, r->data.data(), sizeof(double) * r->data.size());
  return 0;
}

double ref_function_value(const char *name, const double *params, double x0, double y0, double x,
                          double y, int subsampling) {
  FunctionObject *f = make_function(name);
  if (!f) return -1.0;
  f->SetSubsampling(subsampling != 0);
  std::vector<double> p(params, params + f->GetNParams());
  f->Setup(p.data(), 0, x0, y0);
  double v = f->GetValue(x, y);
  delete f;
  return v;
}

double ref_function_total_flux(const char *name, const double *params) {
  FunctionObject *f = make_function(name);
  if (!f) return -1.0;
  std::vector<double> p(params, params + f->GetNParams());
  f->Setup(p.data(), 0, 0.0, 0.0);
  double v = f->CanCalculateTotalFlux() ? f->TotalFlux() : -1.0;
  delete f;
  return v;
}

int ref_use_bootstrap(void *h, unsigned long seed) {
  init_genrand(seed);
  return static_cast<RefModel *>(h)->mo->UseBootstrap();
}

int ref_make_bootstrap_sample(void *h) { return static_cast<RefModel *>(h)->mo->MakeBootstrapSample(); }

// mpfit's own forward-difference Jacobian (solvers/mpfit.cpp:1102-1356),
// obtained by running mpfit with maxiter = 0 is not exposed, so the columns
// are formed here with mp_fdjac2's step rule: h = sqrt(max(epsfcn, MACHEP0))*|x|,
// h = eps when x == 0, one-sided (solvers/mpfit.cpp:1194, 1254-1258).
int ref_fd_jacobian(void *h, const double *params, double *fjac) {
  RefModel *r = static_cast<RefModel *>(h);
  const int n = r->mo->GetNParams();
  const long m = r->mo->GetNDataValues();
  std::vector<double> x(params, params + n), f0(m), f1(m);
  r->mo->ComputeDeviates(f0.data(), x.data());
  const double eps = sqrt(MP_MACHEP0);
  for (int j = 0; j < n; j++) {
    double t = x[j];
    double hh = eps * fabs(t);
    if (hh == 0.0) hh = eps;
    x[j] = t + hh;
    r->mo->ComputeDeviates(f1.data(), x.data());
    x[j] = t;
    for (long i = 0; i < m; i++) fjac[(size_t)j * m + i] = (f1[i] - f0[i]) / hh;
  }
  return 0;
}

// Levenberg-Marquardt fit with the reference's mpfit, configured as
// solvers/levmar_fit.cpp:66-116 does (maxiter, ftol).
int ref_lm_fit(void *h, double *params, const int *fixed, const double *lo, const double *hi,
               double ftol, int maxiter, int *niter, int *nfev, double *chi2, double *chi2_init) {
  RefModel *r = static_cast<RefModel *>(h);
  const int n = r->mo->GetNParams();
  const long m = r->mo->GetNDataValues();
  std::vector<mp_par> pars(n);
  for (int i = 0; i < n; i++) {
    memset(&pars[i], 0, sizeof(mp_par));
    pars[i].fixed = fixed ? fixed[i] : 0;
    if (lo && hi && lo[i] < hi[i]) {
      pars[i].limited[0] = pars[i].limited[1] = 1;
      pars[i].limits[0] = lo[i];
      pars[i].limits[1] = hi[i];
    }
  }
  mp_config cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.maxiter = maxiter;
  cfg.ftol = ftol;
  cfg.verbose = 0;
  mp_result res;
  memset(&res, 0, sizeof(res));
  std::vector<double> xerr(n);
  res.xerror = xerr.data();
  int status = mpfit(fdjac_func, (int)m, n, params, pars.data(), &cfg, r->mo, &res);
  if (niter) *niter = res.niter;
  if (nfev) *nfev = res.nfev;
  if (chi2) *chi2 = res.bestnorm;
  if (chi2_init) *chi2_init = res.orignorm;
  return status;
}

}  // extern "C"
