// The FP32 kick-drift of one single-component site, shared by every FP32
// kernel (register z-march, TMA pipeline, ensemble) so that they all compute
// the same bits.  Rounding is pinned with explicit intrinsics:
//   lap  = sum over the 6 neighbours of (phi_nb - phi) / a^2
//   coef = Mass_Mode M^2 + Lambda_Mode phi^2 / 6 [+ phi^4 / (120 Kappa^2)]
//   pi'  = pi + fk (lap - coef c [- h])          (dynamics.cpp:80-100)
//   phi' = phi + fd pi'                          (dynamics.cpp:183)
// The Laplacian is the reference's (sum of neighbours - 6 phi) / a^2 summed as
// neighbour differences: each difference of two nearby FP32 values is exact
// (Sterbenz), so only the small differences are rounded instead of the O(phi)
// partial sums -- an FP32 trajectory stays about ten times closer to the FP64
// one over 1000 steps, at no cost in memory traffic.
#pragma once

#include "phn_internal.h"

namespace phn {

__device__ __forceinline__ float lap_diff_f32(float c, float xm, float xp, float ym, float yp, float zm, float zp,
                                              float inv_a2) {
  return __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(xp, c), __fsub_rn(xm, c)),
                                       __fadd_rn(__fsub_rn(yp, c), __fsub_rn(ym, c))),
                             __fadd_rn(__fsub_rn(zp, c), __fsub_rn(zm, c))),
                   inv_a2);
}

// Force lap - V'(phi) of a single-component site (l = phi^2) for every
// theory.  Theories 2-5 (dynamics.cpp:109-157) in FP32:
//   2  lap - M sqrt(M) (phi / |phi|) sin(|phi| / sqrt(M))
//   3  the same - M_mono phi
//   4  lap - (Mass_Mode M - g phi / 2 + Lambda_Mode phi^2 / 6) phi
//   5  lap - M phi (1 + phi^2 / M)^(p_mono - 1)
template <int THEORY>
__device__ __forceinline__ float force_f32(const Consts &k, float lap, float c, float l) {
  if (THEORY == 0 || THEORY == 1) {
    float coef = fmaf(l, k.c4_f, k.mmM_f);
    if (THEORY == 0) coef = fmaf(__fmul_rn(l, l), k.c6_f, coef);
    float f = fmaf(-coef, c, lap);
    if (THEORY == 1) f = __fsub_rn(f, k.h_f);
    return f;
  }
  if (THEORY == 2 || THEORY == 3) {
    const float s = sqrtf(l);
    float f = lap;
    if (THEORY == 3) f = fmaf(-k.mmono_f, c, f);
    return fmaf(-(k.m3_f * (c / s)), sinf(s * k.inv_sqrtm_f), f);  // phi = 0 gives 0/0, as in the reference
  }
  if (THEORY == 4) {
    const float coef = fmaf(-k.ghalf_f, c, fmaf(l, k.c4_f, k.mmM_f));
    return fmaf(-coef, c, lap);
  }
  return fmaf(-(k.msq_f * c), powf(fmaf(l, k.inv_m_f, 1.f), k.pm1_f), lap);
}

template <int THEORY>
__device__ __forceinline__ void kick_drift_f32(const Consts &k, float fk, float fd, float c, float xm, float xp,
                                               float ym, float yp, float zm, float zp, float p, float &pn,
                                               float &phin) {
  const float lap = lap_diff_f32(c, xm, xp, ym, yp, zm, zp, k.inv_a2_f);
  const float f = force_f32<THEORY>(k, lap, c, __fmul_rn(c, c));
  pn = fmaf(fk, f, p);
  phin = fmaf(fd, pn, c);
}

}  // namespace phn
