// Per-site terms of the analysis kernels, shared by the island pass and the
// energy-density spectrum: site values of plain, compensated or FP64 fields,
// the BFS summands (islands.cpp:131-198), the energy density rho and Delta
// (fieldanalysis.cpp:437-560).
#pragma once

#include <math.h>

#include <type_traits>

#include "phn_internal.h"

namespace phn {

template <typename T>
__device__ __forceinline__ double val(const T *f, const float *comp, size_t i) {
  double v = (double)f[i];
  if (comp) v -= (double)comp[i];
  return v;
}

// Site values for kernels compiled per storage: KAHAN for compensated FP32
// fields (value = stored - compensation, in FP64), plain otherwise.  The
// choice is a template argument: a runtime test on the compensation pointer
// leaves the FP64 form in the plain kernels (if-converted, it issues for every
// site on GB300's narrow FP64 pipe).
template <bool KAHAN, typename T>
__device__ __forceinline__ double val_k(const T *f, const float *comp, size_t i) {
  if constexpr (KAHAN) return (double)f[i] - (double)comp[i];
  else return (double)f[i];
}

// The same in arithmetic A (FP32 for FP32 storage: no FP64 round trip).
template <typename A, bool KAHAN, typename T>
__device__ __forceinline__ A val_as(const T *f, const float *comp, size_t i) {
  if constexpr (KAHAN) return (A)((double)f[i] - (double)comp[i]);
  else return (A)f[i];
}

// 1/a^2 in arithmetic A: the FP32 kernels take the FP32 constant, so that no
// site converts the FP64 one (a conversion on GB300's narrow FP64 pipe).
template <typename A>
__device__ __forceinline__ A inv_a2_of(const Consts &k) {
  if constexpr (std::is_same<A, float>::value) return k.inv_a2_f;
  else return k.inv_a2;
}

// Potential of one single-component site, theories 0-5: the BFS PotEn
// summand (islands.cpp:137-196), which is also the Interaction summand of
// CalculateVolumeAverages (fieldanalysis.cpp:456-617) for Nc = 1.  The
// expanding box's couplings come folded with the scale factor
// (at_scale_factor); the cosine and power arguments carry it per site.
// (FP64; the constant divisors as products by their reciprocals: these sums
// are compared to the reference's within rounding, not bitwise.)
__device__ __forceinline__ double site_potential(const Consts &k, double c, double c2) {
  const double l2 = c2 * c2;
  const double cos_arg = k.expansion ? sqrt(c2) * k.r_sf_sqrtm : sqrt(c2 * k.r_msq);
  switch (k.theory) {
    case 0:
      return k.mm_half_M * c2 + k.lm * (l2 * k.r_c24) + (l2 * c2 * k.r_c720);
    case 1:
      return k.h * c + k.mm_half_M * c2 + k.lm * (l2 * k.r_c24);
    case 2:
      return k.msq2 * (1. - cos(cos_arg));
    case 3:
      return 0.5 * k.mmono * c2 + k.msq2 * (1. - cos(cos_arg));
    case 4:
      return k.mm_half_M * c2 - k.g * c2 * c * (1.0 / 6.0) + k.lm * (l2 * k.r_c24);
    default:
      return k.t5c * (pow(1. + (k.expansion ? c2 / k.msq_sf2 : c2 * k.r_msq), k.p_mono) - 1.);
  }
}

// The same in FP32, from the FP32 forms of the couplings (those of the FP32
// observation): island statistics of FP32 fields.
__device__ __forceinline__ float site_potential(const Consts &k, float c, float c2) {
  const float l2 = c2 * c2;
  switch (k.theory) {
    case 0:
      return fmaf(k.e6_f, l2 * c2, fmaf(k.e4_f, l2, k.mmh_f * c2));
    case 1:
      return fmaf(k.h_f, c, fmaf(k.e4_f, l2, k.mmh_f * c2));
    case 2:
      return k.msq2_f * (1.f - cosf(sqrtf(c2 * k.inv_m_f)));
    case 3:
      return fmaf(k.mono_half_f, c2, k.msq2_f * (1.f - cosf(sqrtf(c2 * k.inv_m_f))));
    case 4:
      return fmaf(-k.g6_f * c, c2, fmaf(k.e4_f, l2, k.mmh_f * c2));
    default:
      return k.t5c_f * (powf(fmaf(c2, k.inv_m_f, 1.f), k.p_f) - 1.f);
  }
}

// Kinetic summand, with the expanding box's H0/sf terms (islands.cpp:133-138,
// fieldanalysis.cpp:626-629).
__device__ __forceinline__ double site_kinetic(const Consts &k, double c, double p) {
  if (!k.expansion) return 0.5 * (p * p);
  const double hub = k.H0 / k.sf;
  return (0.5 * (p * p) + 0.5 * (hub * hub) * (c * c) - c * p * k.H0 / k.sf);
}

__device__ __forceinline__ float site_kinetic(const Consts &k, float c, float p) {
  if (!k.expansion) return 0.5f * (p * p);
  const float hub = k.hub_f;  // no FP64 per site
  return fmaf(0.5f * (hub * hub) * c, c, fmaf(0.5f * p, p, -c * p * hub));
}

// Per-site energy density: the summand of the reference's Energy
// (fieldanalysis.cpp:437-471,571-579), Nc = 1, in arithmetic A: FP64 for FP64
// fields, FP32 for FP32 fields (their values carry FP32 rounding already; a
// site within that of the threshold is on either side).
template <typename A, bool KAHAN, typename T>
__device__ A site_rho(const T *phi, const float *cphi, const T *pi, const float *cpi, int N, int x, int y, int z,
                      const Consts k) {
  const size_t NN = (size_t)N * N;
  const size_t i = (size_t)z * NN + (size_t)y * N + x;
  const A c = val_as<A, KAHAN>(phi, cphi, i), p = val_as<A, KAHAN>(pi, cpi, i);
  const A fx = val_as<A, KAHAN>(phi, cphi, (size_t)z * NN + (size_t)y * N + (x + 1 == N ? 0 : x + 1));
  const A fy = val_as<A, KAHAN>(phi, cphi, (size_t)z * NN + (size_t)(y + 1 == N ? 0 : y + 1) * N + x);
  const A fz = val_as<A, KAHAN>(phi, cphi, (size_t)(z + 1 == N ? 0 : z + 1) * NN + (size_t)y * N + x);
  const A c2 = c * c;
  const A grad = (((fx - c) * (fx - c) + (fy - c) * (fy - c)) + (fz - c) * (fz - c)) * inv_a2_of<A>(k);
  return site_kinetic(k, c, p) + (A)0.5 * grad + site_potential(k, c, c2);
}

// Half the squared forward differences over a^2 (the BFS GradEn summand,
// islands.cpp:131), with explicit roundings so that every kernel forms it
// alike.
__device__ __forceinline__ float grad_half(float c, float fx, float fy, float fz, float inv_a2) {
  const float dx = __fsub_rn(fx, c), dy = __fsub_rn(fy, c), dz = __fsub_rn(fz, c);
  return __fmul_rn(__fmul_rn(0.5f, __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz))),
                   inv_a2);
}
__device__ __forceinline__ double grad_half(double c, double fx, double fy, double fz, double inv_a2) {
  const double dx = __dsub_rn(fx, c), dy = __dsub_rn(fy, c), dz = __dsub_rn(fz, c);
  return __dmul_rn(__dmul_rn(0.5, __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz))),
                   inv_a2);
}

// Delta (fieldanalysis.cpp:446-560) from the BFS summands of one site:
// kinetic + potential + the full squared differences (twice GradEn's half).
template <typename A>
__device__ __forceinline__ A delta_of(A kin, A grad_h, A pot);
template <>
__device__ __forceinline__ float delta_of(float kin, float grad_h, float pot) {
  return __fadd_rn(__fadd_rn(kin, pot), __fadd_rn(grad_h, grad_h));
}
template <>
__device__ __forceinline__ double delta_of(double kin, double grad_h, double pot) {
  return __dadd_rn(__dadd_rn(kin, pot), __dadd_rn(grad_h, grad_h));
}

// Delta at site (x, y, z) in arithmetic A.
template <typename A, bool KAHAN, typename T>
__device__ A site_delta(const T *phi, const float *cphi, const T *pi, const float *cpi, int N, int x, int y, int z,
                        const Consts k) {
  const size_t NN = (size_t)N * N;
  const size_t i = (size_t)z * NN + (size_t)y * N + x;
  const A c = val_as<A, KAHAN>(phi, cphi, i), p = val_as<A, KAHAN>(pi, cpi, i);
  const A fx = val_as<A, KAHAN>(phi, cphi, (size_t)z * NN + (size_t)y * N + (x + 1 == N ? 0 : x + 1));
  const A fy = val_as<A, KAHAN>(phi, cphi, (size_t)z * NN + (size_t)(y + 1 == N ? 0 : y + 1) * N + x);
  const A fz = val_as<A, KAHAN>(phi, cphi, (size_t)(z + 1 == N ? 0 : z + 1) * NN + (size_t)y * N + x);
  return delta_of<A>(site_kinetic(k, c, p), grad_half(c, fx, fy, fz, inv_a2_of<A>(k)), site_potential(k, c, c * c));
}

}  // namespace phn
