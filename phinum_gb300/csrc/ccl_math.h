// Integer and floating-point shortcuts of the island labelling, shared by
// the kernels (islands.cu) and a host check that compiles this header with
// g++: the same source on both sides.
#pragma once

#ifdef __CUDACC__
#define PHN_HD __host__ __device__
#else
#define PHN_HD
#endif

#include <math.h>

namespace phn {

// Division of site indices (< 2^31) by the lattice edge N without a divide:
// q = umulhi(n, m) >> s with s = floor(log2 N), m = ceil(2^(32+s) / N)
// (Granlund and Montgomery, PLDI 1994).  m < 2^32, and its error e = m N -
// 2^(32+s) < N <= 2^(s+1) makes n e < 2^(32+s) for n < 2^31, so n m / 2^(32+s)
// exceeds n / N by less than 1/N and the floor is exact.  Powers of two
// shift (m = 0).
struct DivN {
  unsigned m;
  int s;
};

inline DivN make_divn(unsigned d) {
  int s = 0;
  while ((2u << s) <= d) ++s;  // floor(log2 d)
  if ((d & (d - 1)) == 0) return DivN{0u, s};
  const unsigned long long num = 1ull << (32 + s);
  return DivN{(unsigned)((num + d - 1) / d), s};
}

PHN_HD inline unsigned div_n(const DivN &q, unsigned n) {
#ifdef __CUDA_ARCH__
  return q.m ? __umulhi(n, q.m) >> q.s : n >> q.s;
#else
  return q.m ? (unsigned)(((unsigned long long)n * q.m) >> 32) >> q.s : n >> q.s;
#endif
}

// The reference mask (islands.cpp:76) Phi^2/2 + Pi^2/2 > thr, evaluated by
// the reference in FP64, decided in FP32 where that is safe.  For FP32 values
// c, p the exact sum S = c^2/2 + p^2/2; s = (c c + RN(p p)) / 2 in one fma is
// within 2^-23 (plus 2^-48) of S relative.  [lo, hi] brackets thr by 2^-19
// relative (each bound rounded to FP32, 2^-24 more): s > hi implies S > thr
// (1 + 2^-20), so RN(S) > thr, and s < lo implies RN(S) < thr.  Thresholds
// outside [2^-100, 2^100] get no bracket (hi = 0: nothing decided in FP32), so
// no FP32 underflow or overflow near the threshold.  NaN compares false both
// ways and falls through.
inline void mask_bracket(double thr, float *lo, float *hi) {
  *lo = 0.f;
  *hi = 0.f;
  if (thr >= 0x1p-100 && thr <= 0x1p100) {
    *lo = (float)(thr * (1.0 - 0x1p-19));
    *hi = (float)(thr * (1.0 + 0x1p-19));
  }
}

// 1 or 0 where the FP32 sum decides the FP64 comparison, -1 elsewhere.
PHN_HD inline int ref_mask_f32(float c, float p, float lo, float hi) {
  const float s = 0.5f * fmaf(c, c, p * p);
  if (hi > 0.f && s > hi) return 1;
  if (hi > 0.f && s < lo) return 0;
  return -1;
}

}  // namespace phn
