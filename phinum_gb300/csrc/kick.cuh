// The FP32 kick-drift of one single-component site, shared by every FP32
// kernel (register z-march, TMA pipeline, ensemble) so that they all compute
// the same bits.  Rounding is pinned with explicit intrinsics:
//   lap  = (((xp + xm) + (yp + ym)) + (zp + zm) - 6 c) / a^2
//   coef = Mass_Mode M^2 + Lambda_Mode phi^2 / 6 [+ phi^4 / (120 Kappa^2)]
//   pi'  = pi + fk (lap - coef c [- h])          (dynamics.cpp:80-100)
//   phi' = phi + fd pi'                          (dynamics.cpp:183)
#pragma once

#include "phn_internal.h"

namespace phn {

template <int THEORY>
__device__ __forceinline__ void kick_drift_f32(const Consts &k, float fk, float fd, float c, float xm, float xp,
                                               float ym, float yp, float zm, float zp, float p, float &pn,
                                               float &phin) {
  const float lap = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(xp, xm), __fadd_rn(yp, ym)), __fadd_rn(zp, zm)),
                                        __fmul_rn(-6.f, c)),
                              k.inv_a2_f);
  const float l = __fmul_rn(c, c);
  float coef = fmaf(l, k.c4_f, k.mmM_f);
  if (THEORY == 0) coef = fmaf(__fmul_rn(l, l), k.c6_f, coef);
  float f = fmaf(-coef, c, lap);
  if (THEORY == 1) f = __fsub_rn(f, k.h_f);
  pn = fmaf(fk, f, p);
  phin = fmaf(fd, pn, c);
}

}  // namespace phn
