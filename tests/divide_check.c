/* Host restatement of the FP64 step kernels' division by per-launch
 * constants (div_by_near / div_by in phinum_gb300/csrc/phn_internal.h),
 * checked against IEEE division; compiled and run by tests/test_divide_host.py.
 * The device code itself is checked on a GPU by phn_divide_selftest.
 *
 *   div_by_near: q = RN(a RN(1/b)), for divisors with |b RN(1/b) - 1| <= 2^-54
 *                (6 Nc, 24 Nc, 120 Nc^2 for Nc <= 4), then one correction
 *                q + RN(a - b q) RN(1/b);
 *   div_by:      q = fma(a, y_h, RN(a y_l)), y_h = RN(1/b),
 *                y_l = RN((1 - b y_h) / b), then the same correction.
 * The kernels take this path for 2^-900 <= |a| < 2^900 and divisors in
 * [2^-100, 2^100]; the operands here cover that range, its edges included,
 * and half of them sit within 2 ulps of a quotient midpoint.
 * Prints one line: divisors, operands, misses. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t st = 0x9E3779B97F4A7C15ull;
static uint64_t xr(void) {
  st ^= st << 13;
  st ^= st >> 7;
  st ^= st << 17;
  return st;
}

/* a double with a random significand and an exponent in [lo_e, hi_e) */
static double rnd_in(int lo_e, int hi_e) {
  const uint64_t m = xr() & ((1ull << 52) - 1);
  const int e = lo_e + (int)(xr() % (uint64_t)(hi_e - lo_e));
  const uint64_t bits = ((uint64_t)(e + 1023) << 52) | m;
  double d;
  memcpy(&d, &bits, 8);
  return (xr() & 1) ? -d : d;
}

static int in_range(double a) { return fabs(a) >= 0x1p-900 && fabs(a) < 0x1p900; }

static double div_near(double a, double b, double rb) {
  const double q = a * rb;
  return fma(fma(-b, q, a), rb, q);
}

static double div_two_word(double a, double b, double yh, double yl) {
  const double q = fma(a, yh, a * yl);
  return fma(fma(-b, q, a), yh, q);
}

int main(int argc, char **argv) {
  const long n = argc > 1 ? atol(argv[1]) : 100000L;
  double bs[96];
  int nb = 0, near_bad = 0;
  const double fixed[] = {sqrt(3.), 720. * 3.0000000000000004, 720. * sqrt(3.) * sqrt(3.), 0.7, 3., 7., 10., 0.49,
                          sqrt(0.49), 9., 1.0363397126425293, 1.7320508075688772 * 1.0363397126425293, 0.0625, 0.07,
                          11., 0x1p-100, 0x1p100, 0x1.fffffffffffffp99, 0x1.0000000000001p-100};
  for (unsigned i = 0; i < sizeof fixed / sizeof fixed[0]; i++) bs[nb++] = fixed[i];
  while (nb < 80) bs[nb++] = fabs(rnd_in(-100, 100));
  /* the near divisors: 6 Nc, 24 Nc, 120 Nc^2 */
  const int first_near = nb;
  for (int nc = 1; nc <= 4; nc++) {
    bs[nb++] = 6.0 * nc;
    bs[nb++] = 24.0 * nc;
    bs[nb++] = 120.0 * nc * nc;
  }
  long bad = 0, done = 0;
  for (int j = 0; j < nb; j++) {
    const double b = bs[j], yh = 1.0 / b, yl = fma(-b, yh, 1.0) / b;
    const int near = j >= first_near;
    if (near && !(fabs(fma(b, yh, -1.0)) <= 0x1p-54)) near_bad++;
    for (long i = 0; i < n; i++) {
      double a;
      const int kind = (int)(i % 4);
      if (kind == 0) {
        a = rnd_in(-900, 900);
      } else if (kind == 1) {
        /* the guard's edges */
        a = (xr() & 1) ? rnd_in(-900, -890) : rnd_in(890, 900);
      } else {
        /* within 2 ulps of b times a quotient midpoint */
        const double q = rnd_in(-700, 700);
        const double up = nextafter(q, INFINITY) - q;
        a = b * (q + 0.5 * up);
        int k = (int)(xr() % 5) - 2;
        for (; k > 0; k--) a = nextafter(a, INFINITY);
        for (; k < 0; k++) a = nextafter(a, -INFINITY);
      }
      if (!in_range(a)) continue;
      done++;
      const double q = near ? div_near(a, b, yh) : div_two_word(a, b, yh, yl);
      if (q != a / b) bad++;
    }
  }
  printf("divisors %d operands %ld misses %ld near_divisors_not_near %d\n", nb, done, bad, near_bad);
  return 0;
}
