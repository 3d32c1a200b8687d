// C ABI: handle lifetime, field transfer, the reference clock and the run
// loop.  The host keeps tau/Last_*_update exactly as dynamics.cpp:28-237 does
// (FP64, same operation order), so the per-step kick and drift factors handed
// to the kernels are the reference's own values.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "phn_internal.h"

namespace {
thread_local char g_err[512] = "";
}

namespace phn {
int set_error(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}
int cuda_error(cudaError_t e, const char *what) {
  if (e == cudaErrorMemoryAllocation) return set_error(PHN_ERR_NOMEM, "%s: %s", what, cudaGetErrorString(e));
  return set_error(PHN_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}
}  // namespace phn

using namespace phn;

#define CK(call)                                         \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_error(e_, #call); \
  } while (0)

int phn::validate_params(const phn_params *p) {
  if (!p) return set_error(PHN_ERR_INVALID, "params is NULL");
  if (p->N < 2 || p->N > 2048) return set_error(PHN_ERR_INVALID, "N=%d outside [2, 2048]", p->N);
  if (p->Nc < 1 || p->Nc > PHN_MAX_NC) return set_error(PHN_ERR_UNSUPPORTED, "Nc=%d outside [1, %d]", p->Nc, PHN_MAX_NC);
  if (p->potential < 0 || p->potential > 5) return set_error(PHN_ERR_INVALID, "theory %d", p->potential);
  if (p->potential >= 2 && !(p->m_sqr > 0.0)) return set_error(PHN_ERR_INVALID, "theory %d needs M_sqr > 0", p->potential);
  if (p->potential == 5 && !(p->p_mono != 0.0)) return set_error(PHN_ERR_INVALID, "p_mono must be non-zero");
  if (p->precision == PHN_FP32_PAIR)
    return set_error(PHN_ERR_UNSUPPORTED, "FP32 pairs serve the adjoint's forward solve only");
  if (p->precision < PHN_FP64 || p->precision > PHN_FP32_KAHAN)
    return set_error(PHN_ERR_INVALID, "precision %d", p->precision);
  if (!(p->a > 0.0) || !isfinite(p->a)) return set_error(PHN_ERR_INVALID, "a must be positive");
  if (!isfinite(p->dt)) return set_error(PHN_ERR_INVALID, "dt must be finite");
  if (p->potential == 0 && !(p->kappa != 0.0)) return set_error(PHN_ERR_INVALID, "Kappa must be non-zero");
  if (p->expanding != 0 && p->expanding != 1) return set_error(PHN_ERR_INVALID, "expansion %d", p->expanding);
  if (p->expanding && !(p->H0 > 0.0 && isfinite(p->H0)))
    return set_error(PHN_ERR_INVALID, "the expanding box needs H_0 > 0");
  if (p->expanding && !(1. + 2. * p->H0 * p->T0 > 0.0))
    return set_error(PHN_ERR_INVALID, "1 + 2 H_0 T0 must be positive");
  return PHN_OK;
}

// RN(1/b) of every constant divisor the FP64 kernels divide by (div_by,
// div_by_near), the low words RN((1 - b RN(1/b))/b) of div_by's two-word
// reciprocals (the residual 1 - b RN(1/b) is exact in one fma), and whether
// all divisors lie in [2^-100, 2^100], where the residual steps cannot
// underflow or overflow for the operands div_by accepts.
static void set_reciprocals(Consts &k) {
  const double divisors[] = {k.six_nc, k.kappa, k.c120, k.c24, k.c720, k.a2, k.sqrt_m, k.msq, k.sf, k.sf_sqrtm};
  double *recips[] = {&k.r_six_nc, &k.r_kappa, &k.r_c120, &k.r_c24, &k.r_c720, &k.r_a2, &k.r_sqrtm, &k.r_msq,
                      &k.r_sf, &k.r_sf_sqrtm};
  double *lows[] = {nullptr, &k.l_kappa, nullptr, nullptr, &k.l_c720, &k.l_a2, &k.l_sqrtm, &k.l_msq,
                    &k.l_sf, &k.l_sf_sqrtm};
  k.fastdiv = 1;
  for (int i = 0; i < 10; ++i) {
    const double b = divisors[i];
    const double m = fabs(b);
    // unused divisors (zero couplings of other theories) get no reciprocal
    if (b == 0.0) {
      *recips[i] = 0.0;
      if (lows[i]) *lows[i] = 0.0;
      continue;
    }
    *recips[i] = 1.0 / b;
    if (lows[i]) *lows[i] = fma(-b, *recips[i], 1.0) / b;
    if (!(m >= 0x1p-100 && m <= 0x1p100)) k.fastdiv = 0;
  }
  // the kernels divide by 6 Nc, 24 Nc and 120 Nc^2 from RN(a RN(1/b))
  // (div_by_near): their reciprocals must be within 2^-54 (b * RN(1/b) - 1
  // is exact in one fma); true for Nc <= 4, checked all the same
  const double near[] = {k.six_nc, k.c24, k.c120};
  for (double b : near)
    if (!(fabs(fma(b, 1.0 / b, -1.0)) <= 0x1p-54)) k.fastdiv = 0;
}

// Coefficients evaluated with the reference's expressions (dynamics.cpp:80-100,
// fieldanalysis.cpp:445-579); see Consts.
Consts phn::make_consts(const phn_params *p) {
  Consts k;
  memset(&k, 0, sizeof(k));
  const int Nc = p->Nc;
  k.N = p->N;
  k.Nc = Nc;
  k.theory = p->potential;
  k.a2 = p->a * p->a;
  {
    int ex = 0;
    k.a2_pow2 = frexp(k.a2, &ex) == 0.5;
    k.inv_a2 = 1.0 / k.a2;
  }
  k.mmM = p->mass_mode * p->m_sqr;
  k.lm = (double)p->lambda_mode;
  k.six_nc = 6. * Nc;
  k.kappa = p->kappa;
  k.c120 = 120. * Nc * Nc;
  k.h = p->h;
  k.mm_half_M = (p->mass_mode) * 0.5 * p->m_sqr;
  k.c24 = 24.0 * Nc;
  k.c720 = 720.0 * Nc * Nc * p->kappa * p->kappa;
  k.inv_a2_f = (float)(1.0 / k.a2);
  k.mmM_f = (float)k.mmM;
  k.c4_f = (float)(k.lm / k.six_nc);
  k.c6_f = p->potential == 0 ? (float)(1.0 / (p->kappa * p->kappa * k.c120)) : 0.f;
  k.h_f = (float)p->h;
  k.mmh_f = (float)k.mm_half_M;
  k.e4_f = (float)(k.lm / k.c24);
  k.e6_f = p->potential == 0 ? (float)(1.0 / k.c720) : 0.f;
  // theories 2-5 (dynamics.cpp:109-157, fieldanalysis.cpp:482-617)
  k.msq = p->m_sqr;
  k.sqrt_m = sqrt(p->m_sqr);
  k.m3 = p->m_sqr * sqrt(p->m_sqr);
  k.msq2 = p->m_sqr * p->m_sqr;
  k.mmono = p->m_mono_sqr;
  k.g = p->g;
  k.p_mono = p->p_mono;
  k.t5c = p->potential == 5 ? k.msq2 * 0.5 / p->p_mono : 0.0;
  k.m3_f = (float)k.m3;
  k.inv_sqrtm_f = p->m_sqr > 0 ? (float)(1.0 / k.sqrt_m) : 0.f;
  k.inv_m_f = p->m_sqr > 0 ? (float)(1.0 / p->m_sqr) : 0.f;
  k.mmono_f = (float)p->m_mono_sqr;
  k.ghalf_f = (float)(p->g / 2.);
  k.msq_f = (float)p->m_sqr;
  k.pm1_f = (float)(p->p_mono - 1);
  k.p_f = (float)p->p_mono;
  k.msq2_f = (float)k.msq2;
  k.mono_half_f = (float)(0.5 * p->m_mono_sqr);
  k.g6_f = (float)(p->g / 6.0);
  k.t5c_f = (float)k.t5c;
  k.expansion = p->expanding;
  k.H0 = p->H0;
  k.sf = 1.0;
  k.sf_sqrtm = k.sqrt_m;
  k.msq_sf2 = k.msq;
  set_reciprocals(k);
  return k;
}

// The couplings the expanding box multiplies by powers of the scale factor
// (dynamics.cpp:88-163, fieldanalysis.cpp:461-615, islands.cpp:136-196),
// each in the reference's left-to-right order.
Consts phn::at_scale_factor(const Consts &k0, double sf) {
  Consts k = k0;
  k.sf = sf;
  k.mmM = k0.mmM * sf * sf;          // Mass_Mode * BareM_sqr*scale_factor*scale_factor
  k.h = k0.h * sf * sf * sf;         // h*scale_factor*scale_factor*scale_factor
  k.m3 = k0.m3 * sf * sf * sf;       // BareM_sqr*sqrt(BareM_sqr)*scale_factor^3
  k.mmono = k0.mmono * sf * sf;      // BareM_mono_sqr * scale_factor*scale_factor
  k.g = k0.g * sf;                   // g*scale_factor
  k.sf_sqrtm = sf * k0.sqrt_m;       // scale_factor*sqrt(BareM_sqr)
  k.msq_sf2 = k0.msq * sf * sf;      // BareM_sqr * scale_factor * scale_factor
  // energy terms
  k.mm_half_M = k0.mm_half_M * sf * sf;
  k.c720 = k0.c720 * sf * sf;
  const double m2 = sf * sf * k0.msq;  // sqr(scale_factor*scale_factor*BareM_sqr)
  k.msq2 = m2 * m2;
  k.t5c = k0.theory == 5 ? k.msq2 * 0.5 / k0.p_mono : 0.0;
  // FP32 forms
  k.hub_f = (float)(k0.H0 / sf);
  k.mmM_f = (float)k.mmM;
  k.c6_f = k0.theory == 0 ? (float)(1.0 / (k0.kappa * k0.kappa * k0.c120 * sf * sf)) : 0.f;
  k.h_f = (float)k.h;
  k.mmh_f = (float)k.mm_half_M;
  k.e6_f = k0.theory == 0 ? (float)(1.0 / k.c720) : 0.f;
  k.m3_f = (float)k.m3;
  k.inv_sqrtm_f = k0.msq > 0 ? (float)(1.0 / k.sf_sqrtm) : 0.f;
  k.inv_m_f = k0.msq > 0 ? (float)(1.0 / k.msq_sf2) : 0.f;
  k.mmono_f = (float)k.mmono;
  k.ghalf_f = (float)(k.g / 2.);
  k.msq_f = (float)k.msq_sf2;
  k.msq2_f = (float)k.msq2;
  k.mono_half_f = (float)(0.5 * k.mmono);
  k.g6_f = (float)(k.g / 6.0);
  k.t5c_f = (float)k.t5c;
  set_reciprocals(k);
  return k;
}

static void free_all(phn_handle *h) {
  if (!h) return;
  spectrum_release(h);
  islands_release(h);
  cudaFree(h->phi[0]);
  cudaFree(h->phi[1]);
  cudaFree(h->pi);
  cudaFree(h->cphi);
  cudaFree(h->cpi);
  cudaFree(h->partials);
  cudaFree(h->fold_groups);
  cudaFree(h->d_avg);
  cudaFree(h->d_ref);
  cudaFree(h->d_err);
  if (h->h_avg) cudaFreeHost(h->h_avg);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

extern "C" {

int phn_abi_version(void) { return PHN_ABI_VERSION; }

const char *phn_last_error(void) { return g_err; }

int phn_device_count(int *count) {
  if (!count) return set_error(PHN_ERR_INVALID, "count is NULL");
  *count = 0;
  cudaError_t e = cudaGetDeviceCount(count);
  if (e != cudaSuccess) {
    *count = 0;
    return cuda_error(e, "cudaGetDeviceCount");
  }
  return PHN_OK;
}

// tau_conformal and scale_factor at cosmic time tau (dynamics.cpp:39-40, :204-205).
static void conformal(phn_handle *h) {
  const double H0 = h->p.H0;
  h->tau_c = (sqrt(1. + 2. * H0 * h->tau) - 1.) / H0;
  h->sf = sqrt(1. + 2. * H0 * h->tau);
}

int phn_reset(phn_handle *h) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  h->tau = h->p.T0;
  h->dtau = h->p.dt * h->p.a;
  h->last_field = h->tau;
  h->last_mom = h->tau;
  if (h->p.expanding) {
    conformal(h);
  } else {
    h->tau_c = h->tau;
    h->sf = 1.0;
  }
  h->last_mom_c = h->tau_c;
  h->last_field_c = h->tau_c;
  h->steps = 0;
  return PHN_OK;
}

int phn_create(const phn_params *params, phn_handle **out) {
  if (!out) return set_error(PHN_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int r = validate_params(params);
  if (r) return r;
  phn_handle *h = new phn_handle();
  memset((void *)h, 0, sizeof(*h));
  h->p = *params;
  h->k = make_consts(params);
  h->grid = lattice_grid(params->N);
  h->V = (size_t)params->N * params->N * params->N;
  h->elem = params->precision == PHN_FP64 ? sizeof(double) : sizeof(float);
  const size_t bytes = h->V * params->Nc * h->elem;
  cudaError_t e = cudaGetDevice(&h->device);
#define CKF(call)                                  \
  do {                                             \
    e = (call);                                    \
    if (e != cudaSuccess) {                        \
      int rr = cuda_error(e, #call);               \
      free_all(h);                                 \
      return rr;                                   \
    }                                              \
  } while (0)
  if (e != cudaSuccess) {
    int rr = cuda_error(e, "cudaGetDevice");
    delete h;
    return rr;
  }
  CKF(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CKF(cudaEventCreate(&h->ev0));
  CKF(cudaEventCreate(&h->ev1));
  CKF(cudaMalloc(&h->phi[0], bytes));
  CKF(cudaMalloc(&h->phi[1], bytes));
  CKF(cudaMalloc(&h->pi, bytes));
  CKF(cudaMemsetAsync(h->phi[0], 0, bytes, h->stream));
  CKF(cudaMemsetAsync(h->phi[1], 0, bytes, h->stream));
  CKF(cudaMemsetAsync(h->pi, 0, bytes, h->stream));
  if (params->precision == PHN_FP32_KAHAN) {
    CKF(cudaMalloc(&h->cphi, bytes));
    CKF(cudaMalloc(&h->cpi, bytes));
    CKF(cudaMemsetAsync(h->cphi, 0, bytes, h->stream));
    CKF(cudaMemsetAsync(h->cpi, 0, bytes, h->stream));
  }
  // default variant from N = 256 up: 8-row tiles, pi streamed from HBM,
  // aligned grid (fewer y-halo re-reads, halo rows served by L2); 4-row
  // tiles below.  phn_autotune can override.
  h->tma_variant = params->N >= 256 ? tma_default_variant(params->N) : 0;
  h->tma_grid = tma_supported(*params) ? tma_grid(*params, h->tma_variant) : 0;
  if (h->tma_grid == 0 && tma_supported(*params)) {
    h->tma_variant = 0;
    h->tma_grid = tma_grid(*params, 0);
  }
  h->path = h->tma_grid > 0 ? PHN_PATH_TMA : PHN_PATH_PLAIN;
  h->x4_variant = 0;
  h->x4_grid = x4_supported(*params) ? x4_grid(*params, 0) : 0;
  h->x4_obs_grid = h->x4_grid > 0 ? x4_grid(*params, x4_obs_variant(0)) : 0;
  {
    int recs = h->grid.nblocks;
    if (h->tma_grid > 0)
      for (int v = 0; v < tma_num_variants(params->N); ++v) {
        const int g = tma_grid(*params, v);
        if (g > recs) recs = g;
      }
    if (h->x4_grid > 0)
      for (int v = 0; v < x4_num_variants(); ++v) {
        const int g = x4_grid(*params, v);
        if (g > recs) recs = g;
      }
    h->partial_cap = recs;
    CKF(cudaMalloc(&h->partials, (size_t)recs * REC * sizeof(double)));
    h->fold_cap = (recs + FIN_GROUP - 1) / FIN_GROUP;
    CKF(cudaMalloc(&h->fold_groups, (size_t)h->fold_cap * REC * sizeof(double)));
  }
  CKF(cudaMalloc(&h->d_err, sizeof(int)));
  CKF(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
  CKF(cudaMalloc(&h->d_avg, sizeof(phn_averages)));
  h->h_avg_cap = 64;
  CKF(cudaHostAlloc((void **)&h->h_avg, h->h_avg_cap * sizeof(phn_averages), cudaHostAllocDefault));
  CKF(cudaStreamSynchronize(h->stream));
#undef CKF
  phn_reset(h);
  *out = h;
  return PHN_OK;
}

int phn_destroy(phn_handle *h) {
  if (!h) return PHN_OK;
  cudaStreamSynchronize(h->stream);
  free_all(h);
  return PHN_OK;
}

static int ensure_ref_staging(phn_handle *h) {
  if (h->d_ref) return PHN_OK;
  const size_t n = (size_t)h->p.Nc * h->p.N * h->p.N * (h->p.N + 2);
  CK(cudaMalloc(&h->d_ref, n * sizeof(double)));
  return PHN_OK;
}

}  // extern "C"

// phn_upload / phn_download for reference-layout arrays of R (double or float).
template <typename R>
static int upload_ref(phn_handle *h, const R *Phi, const R *Pi) {
  if (!h || !Phi || !Pi) return set_error(PHN_ERR_INVALID, "NULL argument");
  int r = ensure_ref_staging(h);
  if (r) return r;
  const int N = h->p.N, Nc = h->p.Nc;
  const size_t n = (size_t)Nc * N * N * (N + 2);
  R *stage = (R *)h->d_ref;  // n doubles of room
  // phi
  CK(cudaMemcpyAsync(stage, Phi, n * sizeof(R), cudaMemcpyHostToDevice, h->stream));
  if (h->p.precision == PHN_FP32_KAHAN)
    CK(launch_from_ref_kahan(stage, (float *)h->phi[h->cur], h->cphi, N, Nc, h->stream));
  else
    CK(launch_from_ref(stage, h->phi[h->cur], h->p.precision, N, Nc, h->stream));
  // pi
  CK(cudaMemcpyAsync(stage, Pi, n * sizeof(R), cudaMemcpyHostToDevice, h->stream));
  if (h->p.precision == PHN_FP32_KAHAN)
    CK(launch_from_ref_kahan(stage, (float *)h->pi, h->cpi, N, Nc, h->stream));
  else
    CK(launch_from_ref(stage, h->pi, h->p.precision, N, Nc, h->stream));
  h->launches += 2;
  CK(cudaStreamSynchronize(h->stream));
  return PHN_OK;
}

template <typename R>
static int download_ref(phn_handle *h, R *Phi, R *Pi) {
  if (!h || (!Phi && !Pi)) return set_error(PHN_ERR_INVALID, "NULL argument");
  int r = ensure_ref_staging(h);
  if (r) return r;
  const int N = h->p.N, Nc = h->p.Nc;
  const size_t n = (size_t)Nc * N * N * (N + 2);
  const bool kahan = h->p.precision == PHN_FP32_KAHAN;
  R *stage = (R *)h->d_ref;
  if (Phi) {
    if (kahan)
      CK(launch_to_ref_kahan((const float *)h->phi[h->cur], h->cphi, stage, N, Nc, h->stream));
    else
      CK(launch_to_ref(h->phi[h->cur], stage, h->p.precision, N, Nc, h->stream));
    CK(cudaMemcpyAsync(Phi, stage, n * sizeof(R), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->launches++;
  }
  if (Pi) {
    // exchange() moves Phi only (comm.cpp:43-61): Pi's ghost slabs are never
    // written by the reference, so only the interior is returned.
    const size_t slab = (size_t)Nc * N * N;
    if (kahan)
      CK(launch_to_ref_kahan((const float *)h->pi, h->cpi, stage, N, Nc, h->stream));
    else
      CK(launch_to_ref(h->pi, stage, h->p.precision, N, Nc, h->stream));
    CK(cudaMemcpyAsync(Pi + slab, stage + slab, slab * N * sizeof(R), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->launches++;
  }
  return PHN_OK;
}

extern "C" {

int phn_upload(phn_handle *h, const double *Phi, const double *Pi) { return upload_ref(h, Phi, Pi); }
int phn_download(phn_handle *h, double *Phi, double *Pi) { return download_ref(h, Phi, Pi); }
int phn_upload_f32(phn_handle *h, const float *Phi, const float *Pi) { return upload_ref(h, Phi, Pi); }
int phn_download_f32(phn_handle *h, float *Phi, float *Pi) { return download_ref(h, Phi, Pi); }

int phn_time(const phn_handle *h, double *tau, int *total_stepcount) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (tau) *tau = h->tau;
  if (total_stepcount) *total_stepcount = h->steps;
  return PHN_OK;
}

int phn_conformal_time(const phn_handle *h, double *tau_conformal, double *scale_factor) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (tau_conformal) *tau_conformal = h->tau_c;
  if (scale_factor) *scale_factor = h->sf;
  return PHN_OK;
}

static int step_once(phn_handle *h, int mode);

// One evolve() of the expanding box (dynamics.cpp:196-213): the kick at
// tau + dtau/2 with that time's scale factor, both factors in conformal time.
// An observation reads the state before the step with the scale factor it
// has, so an observed step is an observation launch and a step launch.
static int step_expanding(phn_handle *h, int mode) {
  if (mode == MODE_STEP_OBS) {
    int r = step_once(h, MODE_OBS);
    return r ? r : step_once(h, MODE_STEP);
  }
  return step_once(h, mode);
}

// One evolve(): host clock as dynamics.cpp:196-237, one fused kernel.
static int step_once(phn_handle *h, int mode) {
  if (h->p.expanding && mode == MODE_STEP_OBS) return step_expanding(h, mode);
  StepF s;
  Consts kx;  // the expanding box's couplings at this launch's scale factor
  const bool ex = h->p.expanding != 0;
  if (mode != MODE_OBS) {
    h->tau += 0.5 * h->dtau;
    if (ex) {
      conformal(h);
      s.fk = h->tau_c - h->last_mom_c;
      kx = at_scale_factor(h->k, h->sf);
    } else {
      s.fk = h->tau - h->last_mom;
    }
    h->last_mom = h->tau;
    h->last_mom_c = ex ? h->tau_c : h->tau;
    h->tau += 0.5 * h->dtau;
    if (ex) {
      conformal(h);
      s.fd = h->tau_c - h->last_field_c;
    } else {
      s.fd = h->tau - h->last_field;
      h->tau_c = h->tau;
    }
    h->last_field = h->tau;
    h->last_field_c = h->tau_c;
  } else {
    s.fk = s.fd = 0.0;
    if (ex) kx = at_scale_factor(h->k, h->sf);
    h->obs_sf = h->sf;
  }
  const Consts &k = ex ? kx : h->k;
  const int nxt = 1 - h->cur;
  cudaError_t e;
  switch (h->p.precision) {
    case PHN_FP64:
      e = launch_step_f64(k, h->grid, mode, (const double *)h->phi[h->cur], (double *)h->phi[nxt],
                          (double *)h->pi, s, h->partials, h->stream);
      if (mode != MODE_STEP) h->obs_records = h->grid.nblocks;
      break;
    case PHN_FP32:
      if (h->path == PHN_PATH_X4) {
        const bool obs = mode != MODE_STEP;
        e = launch_step_f32_x4(k, obs ? x4_obs_variant(h->x4_variant) : h->x4_variant,
                               obs ? h->x4_obs_grid : h->x4_grid, mode, (const float *)h->phi[h->cur],
                               (float *)h->phi[nxt], (float *)h->pi, nullptr, nullptr, s, h->partials, h->stream);
        if (obs) h->obs_records = h->x4_obs_grid;
      } else if (h->path == PHN_PATH_TMA && mode != MODE_OBS) {
        e = launch_step_f32_tma(k, h->tma_variant, h->tma_grid, mode == MODE_STEP_OBS, (const float *)h->phi[h->cur],
                                (float *)h->phi[nxt], (float *)h->pi, s, h->partials, h->d_err, h->stream);
        if (mode == MODE_STEP_OBS) h->obs_records = h->tma_grid;
      } else {
        e = launch_step_f32(k, h->grid, mode, (const float *)h->phi[h->cur], (float *)h->phi[nxt],
                            (float *)h->pi, s, h->partials, h->stream);
        if (mode != MODE_STEP) h->obs_records = h->grid.nblocks;
      }
      break;
    default:
      if (h->path == PHN_PATH_X4) {
        const bool obs = mode != MODE_STEP;
        e = launch_step_f32_x4(k, obs ? x4_obs_variant(h->x4_variant) : h->x4_variant,
                               obs ? h->x4_obs_grid : h->x4_grid, mode, (const float *)h->phi[h->cur],
                               (float *)h->phi[nxt], (float *)h->pi, h->cphi, h->cpi, s, h->partials, h->stream);
        if (obs) h->obs_records = h->x4_obs_grid;
      } else {
        e = launch_step_kahan(k, h->grid, mode, (const float *)h->phi[h->cur], (float *)h->phi[nxt], h->cphi,
                              h->cphi, (float *)h->pi, h->cpi, s, h->partials, h->stream);
        if (mode != MODE_STEP) h->obs_records = h->grid.nblocks;
      }
      break;
  }
  if (e != cudaSuccess) return cuda_error(e, "step kernel launch");
  h->launches++;
  if (mode != MODE_OBS) {
    h->cur = nxt;
    h->steps++;
  }
  return PHN_OK;
}

// Reads (and clears) the device error word of the bounded waits.
static int check_device_error(phn_handle *h) {
  int word = 0;
  CK(cudaMemcpyAsync(&word, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (word) {
    CK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    return set_error(PHN_ERR_TIMEOUT, "a bounded device wait gave up (code %d)", word);
  }
  return PHN_OK;
}

}  // extern "C"

// nsteps plain steps queued on the handle's stream, no synchronisation.
int phn::evolve_async(phn_handle *h, int nsteps) {
  for (int i = 0; i < nsteps; ++i) {
    int r = step_once(h, MODE_STEP);
    if (r) return r;
  }
  return PHN_OK;
}

extern "C" {

int phn_evolve(phn_handle *h, int nsteps) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (nsteps < 0) return set_error(PHN_ERR_INVALID, "nsteps < 0");
  CK(cudaEventRecord(h->ev0, h->stream));
  for (int i = 0; i < nsteps; ++i) {
    int r = step_once(h, MODE_STEP);
    if (r) return r;
  }
  CK(cudaEventRecord(h->ev1, h->stream));
  CK(cudaEventSynchronize(h->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  h->last_ms = ms;
  h->last_steps = nsteps;
  return check_device_error(h);
}

static int fetch_avg(phn_handle *h, phn_averages *dst_host_slot) {
  CK(launch_finalize(h->p.expanding ? at_scale_factor(h->k, h->obs_sf) : h->k, h->partials, h->obs_records,
                     h->d_avg, h->stream, h->fold_groups, h->fold_cap));
  h->launches += (h->obs_records > 4 * FIN_GROUP && (h->obs_records + FIN_GROUP - 1) / FIN_GROUP <= h->fold_cap) ? 2 : 1;
  CK(cudaMemcpyAsync(dst_host_slot, h->d_avg, sizeof(phn_averages), cudaMemcpyDeviceToHost, h->stream));
  return PHN_OK;
}

int phn_volume_averages(phn_handle *h, phn_averages *out) {
  if (!h || !out) return set_error(PHN_ERR_INVALID, "NULL argument");
  int r = step_once(h, MODE_OBS);
  if (r) return r;
  r = fetch_avg(h, &h->h_avg[0]);
  if (r) return r;
  CK(cudaStreamSynchronize(h->stream));
  *out = h->h_avg[0];
  out->t = h->tau;
  if (out->nonfinite > 0) return set_error(PHN_ERR_NONFINITE, "%.0f non-finite field values", out->nonfinite);
  return PHN_OK;
}

int phn_false_vacuum_decayed(const phn_averages *avg, int potential, int *decayed) {
  if (!avg || !decayed) return set_error(PHN_ERR_INVALID, "NULL argument");
  const double v = avg->interaction;
  // fieldanalysis.cpp:889-892 (theories 0, 1, 4)
  *decayed = (potential == 0 || potential == 1 || potential == 4) ? (v < 0 || v != v || v * 0. != 0.) : 0;
  return PHN_OK;
}

int phn_run_loop(phn_handle *h, int nsteps, double tso, phn_averages *rows, int max_rows, int *nrows) {
  if (!h || nsteps < 0 || (max_rows > 0 && !rows)) return set_error(PHN_ERR_INVALID, "bad argument");
  if (max_rows > h->h_avg_cap) {
    cudaFreeHost(h->h_avg);
    h->h_avg = nullptr;
    h->h_avg_cap = max_rows;
    CK(cudaHostAlloc((void **)&h->h_avg, (size_t)max_rows * sizeof(phn_averages), cudaHostAllocDefault));
  }
  phn_reset(h);
  double last_so = 0.0;
  int n = 0, due_total = 0;
  double *stamps = new double[max_rows > 0 ? max_rows : 1];
  CK(cudaEventRecord(h->ev0, h->stream));
  for (int count = 0; count < nsteps; ++count) {
    // Print_AveragesExtrema cadence (fieldanalysis.cpp:753-780)
    bool due = false;
    if (h->steps == 0) {
      last_so = h->tau;
      due = true;
    } else if (!(h->tau < last_so + tso)) {
      if (h->tau >= last_so + tso) last_so += tso;
      due = true;
    }
    int r;
    if (due) {
      due_total++;
      r = step_once(h, MODE_STEP_OBS);
      if (!r && n < max_rows) {
        r = fetch_avg(h, &h->h_avg[n]);
        stamps[n] = last_so;
        n++;
      }
    } else {
      r = step_once(h, MODE_STEP);
    }
    if (r) {
      delete[] stamps;
      return r;
    }
  }
  cudaError_t e = cudaEventRecord(h->ev1, h->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(h->ev1);
  if (e != cudaSuccess) {
    delete[] stamps;
    return cuda_error(e, "run loop");
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  h->last_steps = nsteps;
  int nonfinite = 0;
  for (int i = 0; i < n; ++i) {
    rows[i] = h->h_avg[i];
    rows[i].t = stamps[i];
    if (rows[i].nonfinite > 0) nonfinite = 1;
  }
  delete[] stamps;
  if (nrows) *nrows = due_total;
  {
    int r = check_device_error(h);
    if (r) return r;
  }
  if (due_total > max_rows) return set_error(PHN_ERR_TRUNCATED, "%d rows due, %d written", due_total, max_rows);
  if (nonfinite) return set_error(PHN_ERR_NONFINITE, "non-finite field values in a row");
  return PHN_OK;
}

int phn_set_path(phn_handle *h, int path) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (path == PHN_PATH_AUTO) path = h->tma_grid > 0 ? PHN_PATH_TMA : PHN_PATH_PLAIN;
  if (path != PHN_PATH_PLAIN && path != PHN_PATH_TMA && path != PHN_PATH_X4)
    return set_error(PHN_ERR_INVALID, "path %d", path);
  if (path == PHN_PATH_TMA && h->tma_grid == 0)
    return set_error(PHN_ERR_UNSUPPORTED, "TMA step needs FP32, Nc = 1, N in {128,256,384,512,768,1024}");
  if (path == PHN_PATH_X4 && h->x4_grid == 0)
    return set_error(PHN_ERR_UNSUPPORTED, "x4 step needs FP32, Nc = 1, N a multiple of 32");
  h->path = path;
  return PHN_OK;
}

// Variants of the FP32 step on this handle: the TMA kernel's, then the x4
// kernel's.
static int n_tma_variants(const phn_handle *h) { return h->tma_grid > 0 ? tma_num_variants(h->p.N) : 0; }
static int n_x4_variants(const phn_handle *h) { return h->x4_grid > 0 ? x4_num_variants() : 0; }

// Selects combined variant v (-1: the plain kernel); returns its grid, 0 if it
// does not apply to this lattice or device.
static int select_variant(phn_handle *h, int v) {
  if (v < 0) {
    h->path = PHN_PATH_PLAIN;
    return h->grid.nblocks;
  }
  const int nt = n_tma_variants(h);
  if (v < nt) {
    const int g = tma_grid(h->p, v);
    if (g > 0) {
      h->path = PHN_PATH_TMA;
      h->tma_variant = v;
      h->tma_grid = g;
    }
    return g;
  }
  const int g = x4_grid(h->p, v - nt);
  const int go = g > 0 ? x4_grid(h->p, x4_obs_variant(v - nt)) : 0;
  if (g > 0 && go > 0) {
    h->path = PHN_PATH_X4;
    h->x4_variant = v - nt;
    h->x4_grid = g;
    h->x4_obs_grid = go;
    return g;
  }
  return 0;
}

int phn_autotune(phn_handle *h, int steps, int *variant, double *best_ms) {
  if (!h || steps < 1) return set_error(PHN_ERR_INVALID, "bad argument");
  const int nt = n_tma_variants(h), nv = nt + n_x4_variants(h);
  if (h->p.precision == PHN_FP64 || nv == 0) {
    if (variant) *variant = -1;
    if (best_ms) *best_ms = 0.0;
    return PHN_OK;  // one kernel only: nothing to choose
  }
  int r = ensure_ref_staging(h);
  if (r) return r;
  // pi (and, compensated, both compensation words) are updated in place by a
  // step: keep copies and put them back after each trial, so the lattice
  // state is unchanged by tuning (phi[cur] is only read)
  const size_t bytes = h->V * h->elem;
  const bool kahan = h->p.precision == PHN_FP32_KAHAN;
  const StepF s = {h->dtau, h->dtau};
  const int path0 = h->path, tv0 = h->tma_variant, xv0 = h->x4_variant;
  const int tg0 = h->tma_grid, xg0 = h->x4_grid, xo0 = h->x4_obs_grid;
  double best = 1e30;
  int best_v = -2;
  float *save_c = nullptr;
  if (kahan) CK(cudaMallocAsync((void **)&save_c, 2 * bytes, h->stream));
  CK(cudaMemcpyAsync(h->d_ref, h->pi, bytes, cudaMemcpyDeviceToDevice, h->stream));
  if (kahan) {
    CK(cudaMemcpyAsync(save_c, h->cphi, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync((char *)save_c + bytes, h->cpi, bytes, cudaMemcpyDeviceToDevice, h->stream));
  }
  // two rounds over the candidates (plain kernel = -1), each keeping its best round
  for (int round = 0; round < 2; ++round)
    for (int v = -1; v < nv; ++v) {
      if (select_variant(h, v) <= 0) continue;
      for (int i = 0; i < steps + 2; ++i) {
        if (i == 2) CK(cudaEventRecord(h->ev0, h->stream));
        cudaError_t e;
        if (h->path == PHN_PATH_TMA)
          e = launch_step_f32_tma(h->k, h->tma_variant, h->tma_grid, false, (const float *)h->phi[h->cur],
                                  (float *)h->phi[1 - h->cur], (float *)h->pi, s, h->partials, h->d_err, h->stream);
        else if (h->path == PHN_PATH_X4)
          e = launch_step_f32_x4(h->k, h->x4_variant, h->x4_grid, MODE_STEP, (const float *)h->phi[h->cur],
                                 (float *)h->phi[1 - h->cur], (float *)h->pi, kahan ? h->cphi : nullptr,
                                 kahan ? h->cpi : nullptr, s, h->partials, h->stream);
        else if (kahan)
          e = launch_step_kahan(h->k, h->grid, MODE_STEP, (const float *)h->phi[h->cur], (float *)h->phi[1 - h->cur],
                                h->cphi, h->cphi, (float *)h->pi, h->cpi, s, h->partials, h->stream);
        else
          e = launch_step_f32(h->k, h->grid, MODE_STEP, (const float *)h->phi[h->cur], (float *)h->phi[1 - h->cur],
                              (float *)h->pi, s, h->partials, h->stream);
        if (e != cudaSuccess) return cuda_error(e, "step kernel launch (autotune)");
        h->launches++;
      }
      CK(cudaEventRecord(h->ev1, h->stream));
      CK(cudaEventSynchronize(h->ev1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
      CK(cudaMemcpyAsync(h->pi, h->d_ref, bytes, cudaMemcpyDeviceToDevice, h->stream));
      if (kahan) {
        CK(cudaMemcpyAsync(h->cphi, save_c, bytes, cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(h->cpi, (char *)save_c + bytes, bytes, cudaMemcpyDeviceToDevice, h->stream));
      }
      if (ms / steps < best) {
        best = ms / steps;
        best_v = v;
      }
    }
  if (save_c) CK(cudaFreeAsync(save_c, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  r = check_device_error(h);
  if (r) return r;
  if (best_v == -2) {  // nothing ran: keep the previous choice
    h->path = path0;
    h->tma_variant = tv0;
    h->x4_variant = xv0;
    h->tma_grid = tg0;
    h->x4_grid = xg0;
    h->x4_obs_grid = xo0;
    return set_error(PHN_ERR_UNSUPPORTED, "no step kernel fits this device");
  }
  select_variant(h, best_v);
  if (variant) *variant = best_v;
  if (best_ms) *best_ms = best;
  return PHN_OK;
}

int phn_set_variant(phn_handle *h, int variant) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  const int nv = n_tma_variants(h) + n_x4_variants(h);
  if (nv == 0) return set_error(PHN_ERR_UNSUPPORTED, "no kernel variants on this handle");
  if (variant < 0 || variant >= nv) return set_error(PHN_ERR_INVALID, "variant %d", variant);
  const int path0 = h->path;
  if (select_variant(h, variant) <= 0) {
    h->path = path0;
    return set_error(PHN_ERR_UNSUPPORTED, "variant %d does not fit this lattice or device", variant);
  }
  return PHN_OK;
}

int phn_num_variants(const phn_handle *h, int *n) {
  if (!h || !n) return set_error(PHN_ERR_INVALID, "NULL argument");
  *n = n_tma_variants(h) + n_x4_variants(h);
  return PHN_OK;
}

int phn_get_path(const phn_handle *h, int *path) {
  if (!h || !path) return set_error(PHN_ERR_INVALID, "NULL argument");
  *path = h->path;
  return PHN_OK;
}

int phn_device_fields(phn_handle *h, void **phi, void **pi, void **stream) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (phi) *phi = h->phi[h->cur];
  if (pi) *pi = h->pi;
  if (stream) *stream = (void *)h->stream;
  return PHN_OK;
}

int phn_synchronize(phn_handle *h) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  CK(cudaStreamSynchronize(h->stream));
  return PHN_OK;
}

int phn_stats(const phn_handle *h, long long *kernel_launches, double *last_evolve_ms, int *last_evolve_steps) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (kernel_launches) *kernel_launches = h->launches;
  if (last_evolve_ms) *last_evolve_ms = h->last_ms;
  if (last_evolve_steps) *last_evolve_steps = h->last_steps;
  return PHN_OK;
}

int phn_pin_host(void *ptr, size_t bytes) {
  if (!ptr || !bytes) return set_error(PHN_ERR_INVALID, "bad argument");
  CK(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
  return PHN_OK;
}

int phn_unpin_host(void *ptr) {
  if (!ptr) return set_error(PHN_ERR_INVALID, "bad argument");
  CK(cudaHostUnregister(ptr));
  return PHN_OK;
}

}  // extern "C"
