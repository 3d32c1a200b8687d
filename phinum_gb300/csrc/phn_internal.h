// Internal declarations shared by the CUDA translation units of libphinum_gpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/phinum_gpu.h"

namespace phn {

// Block shape of the lattice kernels: 32 x-sites (one warp) by 8 y-rows,
// each thread marching a chunk of z-planes.
constexpr int TX = 32;
constexpr int TY = 8;
constexpr int THREADS = TX * TY;

// Observation record written per block by the step kernels and folded by
// finalize_averages.  Sums are FP64.
enum {
  S_PHI = 0,   // [PHN_MAX_NC]
  S_PI = 4,    // [PHN_MAX_NC]
  S_PHI2 = 8,
  S_PI2,
  S_PHIPI,
  S_PHI4,
  S_PHI6,
  S_GRAD,
  S_INTER,
  S_NONFINITE,
  NSUM,        // 16
  E_MIN_V = NSUM,
  E_MIN_I,
  E_MAX_V,
  E_MAX_I,
  E_ABS_V,
  E_ABS_I,
  REC = 24     // doubles per block record (padded)
};
constexpr int FIN_GROUP = 256;  // block records per first-level fold (launch_finalize)


// Coefficients of the kick, the volume averages and the energy density,
// evaluated on the host with the reference's own expressions so that the FP64
// kernels combine exactly the same IEEE values.
struct Consts {
  int N, Nc, theory;
  int a2_pow2;       // sqr(a_t) is a power of two: x / a2 == x * inv_a2 exactly
  double a2;         // sqr(a_t)
  double inv_a2;     // 1 / sqr(a_t)
  double mmM;        // Mass_Mode * BareM_sqr_long
  double lm;         // (double)Lambda_Mode
  double six_nc;     // 6.*Nc
  double kappa;      // Kappa
  double c120;       // 120.*Nc*Nc
  double h;          // h
  double mm_half_M;  // (Mass_Mode)*0.5*BareM_sqr_long
  double c24;        // 24.0*Nc
  double c720;       // 720.0*Nc*Nc*Kappa*Kappa
  // FP32 forms of the kick
  float inv_a2_f, mmM_f, c4_f, c6_f, h_f;
  float hub_f;  // H0 / scale factor (the expanding box's kinetic terms; 0 for the static box)
  // FP32 forms of the energy density
  float mmh_f, e4_f, e6_f;
  // theories 2-5 (Nc = 1): M = BareM_sqr, as the reference writes the terms
  double msq, sqrt_m, m3;  // M, sqrt(M), M sqrt(M)
  double msq2;             // sqr(M)
  double mmono, g, p_mono; // BareM_mono_sqr, g, p_mono
  double t5c;              // sqr(M) * 0.5 / p_mono
  float m3_f, inv_sqrtm_f, inv_m_f, mmono_f, ghalf_f, msq_f, pm1_f, p_f;
  float msq2_f, mono_half_f, g6_f, t5c_f;
  // the expanding box (dynamics.cpp:88-163, fieldanalysis.cpp:461-629): a
  // launch's Consts are those of make_consts folded with one scale factor by
  // at_scale_factor; the fields below let the FP64 kernels keep the per-site
  // divisions by sf that the reference writes
  int expansion;
  double H0;
  double sf;        // scale factor (1 when static)
  double sf_sqrtm;  // sf * sqrt(M)
  double msq_sf2;   // (M sf) sf
  // reciprocals RN(1/b) of the FP64 kernels' constant divisors (div_by,
  // div_by_near) and, for div_by's divisors, the low word l = RN((1 - b r)/b)
  // of a two-word reciprocal r + l; fastdiv = 0 when a divisor lies outside
  // [2^-100, 2^100] or one of 6 Nc, 24 Nc, 120 Nc^2 has a reciprocal further
  // than 2^-54 from 1/b
  int fastdiv;
  double r_six_nc, r_kappa, r_c120, r_c24, r_c720, r_a2, r_sqrtm, r_msq, r_sf, r_sf_sqrtm;
  double l_kappa, l_c720, l_a2, l_sqrtm, l_msq, l_sf, l_sf_sqrtm;
};

// Consts of the expanding box at scale factor sf: every coupling that the
// reference multiplies by powers of sf as a whole (Mass_Mode M sf sf, h sf^3,
// M sqrt(M) sf^3, M_mono sf sf, g sf, and the energy terms) is evaluated once
// here in the reference's left-to-right order, so the FP64 kick that uses them
// stays bit-identical; the FP32 constants are folded the same way.
Consts at_scale_factor(const Consts &k0, double sf);

// a / b, correctly rounded, for a divisor b fixed per launch, from its
// reciprocal rb = RN(1/b) computed on the host.  From a faithful quotient q
// (within one ulp of a/b) and rb = RN(1/b), one correction
// q' = RN(q + RN(a - b q) rb) returns RN(a/b) (Markstein's theorem: P.
// Markstein, IBM J. Res. Dev. 34(1), 1990; M. Cornea-Hasegan, R. Golliver,
// P. Markstein, ARITH-14, 1999), and the fma residual of a faithful quotient
// is exact.  The faithful q comes from
//   div_by_near: q = RN(a rb), for divisors with |b rb - 1| <= 2^-54 (a rb is
//                then within half an ulp of a/b): 6 Nc, 24 Nc, 120 Nc^2,
//                checked on the host;
//   div_by:      q = RN(a rb + RN(a rl)) with the two-word reciprocal rb + rl
//                (rl = RN((1 - b rb)/b), within ~2^-105 of 1/b together), for
//                every other divisor.
// The theorem needs no underflow or overflow in the residuals: operands
// outside 2^-900 <= |a| < 2^900 (zeros, subnormals, infinities, NaN; an
// integer test of the exponent) and handles whose divisors leave
// [2^-100, 2^100] (fastdiv = 0) take IEEE division.  Three or four FP64
// operations instead of a full division: the FP64 kernels are bound by
// GB300's FP64 rate.
__device__ __forceinline__ bool div_fast_range(const Consts &k, double a) {
  const unsigned hi = (unsigned)__double2hiint(a) & 0x7fffffffu;
  return k.fastdiv && hi >= 0x07b00000u && hi < 0x78300000u;
}

__device__ __forceinline__ double div_by_near(const Consts &k, double a, double b, double rb) {
  if (!div_fast_range(k, a)) return a / b;
  const double q = __dmul_rn(a, rb);
  return __fma_rn(__fma_rn(-b, q, a), rb, q);
}

__device__ __forceinline__ double div_by(const Consts &k, double a, double b, double rb, double rl) {
  if (!div_fast_range(k, a)) return a / b;
  const double q = __fma_rn(a, rb, __dmul_rn(a, rl));
  return __fma_rn(__fma_rn(-b, q, a), rb, q);
}

// x / sqr(a_t) in IEEE arithmetic.  When sqr(a_t) is a power of two the
// quotient is an exact scaling and the product by its reciprocal rounds the
// same real number the same way (bit-identical, cheaper on the FP64 pipes).
__device__ __forceinline__ double div_a2(const Consts &k, double x) {
  return k.a2_pow2 ? __dmul_rn(x, k.inv_a2) : div_by(k, x, k.a2, k.r_a2, k.l_a2);
}

// Per-step kick and drift factors: tau - Last_Momenta_update and
// tau - Last_Field_update (dynamics.cpp:84,183).
struct StepF {
  double fk, fd;
};

enum StepMode { MODE_STEP = 0, MODE_STEP_OBS = 1, MODE_OBS = 2 };

struct Grid {
  dim3 grid, block;
  int cz;          // z-planes per block
  int nblocks;     // grid.x * grid.y * grid.z
};
Grid lattice_grid(int N);

// Launchers (leapfrog.cu).  Return cudaGetLastError().
cudaError_t launch_step_f64(const Consts &k, const Grid &g, int mode, const double *phi, double *phi_out,
                            double *pi, StepF s, double *partials, cudaStream_t st);
cudaError_t launch_step_f32(const Consts &k, const Grid &g, int mode, const float *phi, float *phi_out,
                            float *pi, StepF s, double *partials, cudaStream_t st);
cudaError_t launch_step_kahan(const Consts &k, const Grid &g, int mode, const float *phi, float *phi_out,
                              const float *cphi, float *cphi_out, float *pi, float *cpi, StepF s,
                              double *partials, cudaStream_t st);
cudaError_t launch_finalize(const Consts &k, const double *partials, int nblocks, phn_averages *out,
                            cudaStream_t st, double *groups = nullptr, int groups_cap = 0);

// TMA-pipelined FP32 step (leapfrog_tma.cu): Nc = 1, N in {128,256,384,512,768,1024};
// variants are tile heights / stage counts, all bit-identical.
bool tma_supported(const phn_params &p);
int tma_num_variants(int N);
int tma_default_variant(int N);
int tma_grid(const phn_params &p, int variant);
cudaError_t launch_step_f32_tma(const Consts &k, int variant, int grid, bool obs, const float *phi, float *phi_out,
                                float *pi, StepF s, double *partials, int *err, cudaStream_t st);

// Register FP32 step with four x-sites per thread (leapfrog_x4.cu): Nc = 1,
// N a multiple of 32, FP32 or compensated FP32 (cphi, cpi non-null);
// variants are block shapes and grid policies, all bit-identical to the
// other kernels of the same precision.  mode: MODE_STEP/STEP_OBS/OBS.
bool x4_supported(const phn_params &p);
int x4_num_variants();
int x4_obs_variant(int variant);  // the persistent variant observation steps use
int x4_grid(const phn_params &p, int variant);
cudaError_t launch_step_f32_x4(const Consts &k, int variant, int grid, int mode, const float *phi, float *phi_out,
                               float *pi, float *cphi, float *cpi, StepF s, double *partials, cudaStream_t st);

// Leapfrog in FP32 pairs (double-float arithmetic; pair.cu), theories 0 and 1,
// Nc = 1, static box: pi (qh, ql) updated in place, phi (ph, pl) -> (oh, ol).
cudaError_t launch_step_pair(const Consts &k, double fk, double fd, const float *ph, const float *pl, float *qh,
                             float *ql, float *oh, float *ol, cudaStream_t st);
cudaError_t launch_pair_from_ref(const double *ref, float *hi, float *lo, int N, cudaStream_t st);
cudaError_t launch_pair_to_f64(const float *hi, const float *lo, double *out, int N, cudaStream_t st);

// Layout conversion between the reference layout (host order, ghosts; R =
// double or float, the reference's pseudo_double) and the device SoA layout
// [a][z][y][x] (layout.cu).
template <typename R>
cudaError_t launch_from_ref(const R *ref, void *dst, int prec, int N, int Nc, cudaStream_t st);
template <typename R>
cudaError_t launch_to_ref(const void *src, R *ref, int prec, int N, int Nc, cudaStream_t st);
template <typename R>
cudaError_t launch_to_ref_kahan(const float *hi, const float *comp, R *ref, int N, int Nc, cudaStream_t st);
template <typename R>
cudaError_t launch_from_ref_kahan(const R *ref, float *hi, float *comp, int N, int Nc, cudaStream_t st);

// Error text for phn_last_error (api.cu).
int set_error(int code, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);

// Parameter checks and kernel coefficients of phn_create (api.cu).
int validate_params(const phn_params *p);
Consts make_consts(const phn_params *p);

}  // namespace phn

// The handle behind the opaque phn_handle pointer.
struct phn_handle {
  phn_params p;
  phn::Consts k;
  phn::Grid grid;
  int device;
  cudaStream_t stream;
  size_t V;            // sites per component
  size_t elem;         // bytes per field element
  void *phi[2];        // double-buffered phi
  void *pi;
  float *cphi, *cpi;   // compensation terms (PHN_FP32_KAHAN)
  int cur;             // phi[cur] holds the current field
  int path;            // PHN_PATH_* in use for FP32 steps
  int tma_grid;        // persistent grid of the TMA step kernel (0: unsupported)
  int tma_variant;     // TMA kernel variant in use (phn_autotune picks it)
  int x4_grid;         // grid of the x4 step kernel (0: unsupported)
  int x4_variant;      // x4 kernel variant in use
  int x4_obs_grid;     // grid of its observation-step variant
  int partial_cap;     // block records the partials buffer holds
  int obs_records;     // block records written by the last observation launch
  double obs_sf;       // scale factor of the state the last observation read
  int *d_err;          // device error word of bounded waits (0: none)
  double *partials;    // block records of the fused observation
  double *fold_groups; // first-level folds of many records (launch_finalize)
  int fold_cap;        // group records fold_groups holds
  phn_averages *d_avg; // finalize output (device)
  phn_averages *h_avg; // pinned host mirror, one per row slot
  int h_avg_cap;
  double *d_ref;       // reference-layout staging for upload/download
  // reference clock (dynamics.cpp:8-50); the expanding box's conformal time,
  // scale factor and conformal update stamps (tau_c = tau, sf = 1 when static)
  double tau, dtau, last_mom, last_field;
  double tau_c, sf, last_mom_c, last_field_c;
  int steps;
  // accounting
  long long launches;
  cudaEvent_t ev0, ev1;
  double last_ms;
  int last_steps;
  // spectrum (spectrum.cu)
  void *spec;
  // islands (islands.cu)
  void *isl;
};

namespace phn {
// The Consts of the handle's current state: folded with its scale factor for
// the expanding box.
inline Consts consts_now(const phn_handle *h) { return h->p.expanding ? at_scale_factor(h->k, h->sf) : h->k; }
void spectrum_release(phn_handle *h);
void islands_release(phn_handle *h);
int islands_labels_mapped(phn_handle *h, const int *map, int n, int *labels);  // islands.cu
int evolve_async(phn_handle *h, int nsteps);  // api.cu: steps queued, no sync
}  // namespace phn
