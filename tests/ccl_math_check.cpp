// Host check of the island labelling's shortcuts (phinum_gb300/csrc/ccl_math.h),
// compiled by tests/test_ccl_math.py: the same header the kernels include.
//   divn:   div_n(make_divn(d), n) == n / d for every edge d in [1, 4096] and
//           sampled n < 2^31 (with the multiples of d and their neighbours);
//   bracket: wherever ref_mask_f32 decides, it agrees with the reference's
//           FP64 test RN(RN(c c) 0.5 + RN(p p) 0.5) > thr, over random fields,
//           thresholds placed within a few ulps of the sum, and special values.
// Prints one line per check with its count of disagreements.
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "ccl_math.h"

using namespace phn;

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;
static uint64_t next_u64() {  // splitmix64
  uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double unit() { return (double)(next_u64() >> 11) * 0x1p-53; }

static bool ref_mask64(float c, float p, double thr) {
  const double cd = c, pd = p;
  const double a = (cd * cd) * 0.5, b = (pd * pd) * 0.5;
  return a + b > thr;
}

static float from_bits(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

int main() {
  long long bad = 0, checked = 0;
  for (unsigned d = 1; d <= 4096; ++d) {
    const DivN q = make_divn(d);
    const unsigned top = 0x7fffffffu / d;
    const unsigned qs[] = {0u, 1u, 2u, 1000u, top / 2, top - 1, top};
    for (unsigned k : qs)
      for (int r = -1; r <= 1; ++r) {
        const long long n = (long long)k * d + r;
        if (n < 0 || n > 0x7fffffffll) continue;
        ++checked;
        if (div_n(q, (unsigned)n) != (unsigned)n / d) ++bad;
      }
    for (int t = 0; t < 256; ++t) {
      const unsigned n = (unsigned)(next_u64() & 0x7fffffffu);
      ++checked;
      if (div_n(q, n) != n / d) ++bad;
    }
  }
  {
    const unsigned n = 0x7fffffffu;
    for (unsigned d = 1; d <= 4096; ++d, ++checked)
      if (div_n(make_divn(d), n) != n / d) ++bad;
  }
  printf("divn checked %lld mismatches %lld\n", checked, bad);

  long long decided = 0, wrong = 0, total = 0, far_total = 0, far_decided = 0;
  auto check = [&](float c, float p, double thr) {
    float lo, hi;
    mask_bracket(thr, &lo, &hi);
    const int dec = ref_mask_f32(c, p, lo, hi);
    ++total;
    if (dec < 0) return false;
    ++decided;
    if ((dec == 1) != ref_mask64(c, p, thr)) ++wrong;
    return true;
  };
  for (int t = 0; t < 4000000; ++t) {
    // fields of every magnitude in [2^-60, 2^60], either sign
    const float c = (float)((unit() - 0.5) * __builtin_ldexp(1.0, (int)(next_u64() % 121) - 60));
    const float p = (float)((unit() - 0.5) * __builtin_ldexp(1.0, (int)(next_u64() % 121) - 60));
    const double cd = c, pd = p;
    const double s = (cd * cd) * 0.5 + (pd * pd) * 0.5;
    // a threshold at the sum, a few ulps off it, a little off it, and random
    double thr = s;
    const int mode = (int)(next_u64() % 4);
    if (mode == 1) {
      const int k = (int)(next_u64() % 9) - 4;
      thr = s;
      for (int j = 0; j < (k < 0 ? -k : k); ++j) thr = k < 0 ? nextafter(thr, 0.0) : nextafter(thr, 1e300);
    } else if (mode == 2) {
      thr = s * (1.0 + (unit() - 0.5) * 0x1p-17);
    } else if (mode == 3) {
      thr = unit() * __builtin_ldexp(1.0, (int)(next_u64() % 241) - 120);
    }
    const bool dec = check(c, p, thr);
    if (mode == 3 && thr >= 0x1p-100 && thr <= 0x1p100) {
      far_total++;
      far_decided += dec;
    }
  }
  // special values: zeros, subnormals, infinities, NaN, the largest floats
  const uint32_t specials[] = {0x00000000u, 0x80000000u, 0x00000001u, 0x007fffffu, 0x00800000u, 0x7f7fffffu,
                               0x7f800000u, 0xff800000u, 0x7fc00000u, 0x3f800000u, 0x5f800000u, 0x1f800000u};
  const double thrs[] = {0.0, 0x1p-120, 0x1p-100, 1e-10, 0.5, 1.0, 49.5, 1e20, 0x1p100, 0x1p120};
  for (uint32_t a : specials)
    for (uint32_t b : specials)
      for (double thr : thrs) check(from_bits(a), from_bits(b), thr);
  printf("bracket checked %lld decided %lld wrong %lld\n", total, decided, wrong);
  printf("random thresholds %lld decided %lld\n", far_total, far_decided);
  return 0;
}
