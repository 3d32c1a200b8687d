/*
 * Single-rank stand-in for the FFTW3-MPI subset that PhiNum's clusterfft.cpp
 * uses (plans at clusterfft.cpp:45-46, execute at :211,248).
 *
 * TEST INFRASTRUCTURE ONLY: it lets the reference's own sources compile
 * unchanged into the oracle library under oracle/_ref/.  FFTW itself is not
 * vendored in the reference and is absent here; this header computes the same
 * unnormalised transforms from the DFT definition:
 *
 *   r2c:  out[k0][k1][k2] = sum_j in[j0][j1][j2] exp(-2 pi i (k0 j0/n0 + k1 j1/n1 + k2 j2/n2)),
 *         0 <= k2 <= n2/2, real input padded to 2*(n2/2+1) in the last dimension;
 *   c2r:  the inverse direction with exp(+2 pi i ...), Hermitian completion of
 *         the last dimension, real output padded the same way, no 1/n factor.
 *
 * One-dimensional passes use an iterative radix-2 FFT when the length is a
 * power of two and a direct O(n^2) sum otherwise; twiddles are evaluated as
 * long double sin/cos of 2 pi k / n.  With one rank the "local" slab is the
 * whole lattice.
 */
#ifndef PHN_ORACLE_FFTW3_MPI_SHIM_H
#define PHN_ORACLE_FFTW3_MPI_SHIM_H

#include <complex>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <vector>

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef long double fftwl_complex[2];

#define FFTW_MEASURE 0U
#define FFTW_ESTIMATE (1U << 6)

namespace phn_fft_shim {

struct PlanBase {
  virtual ~PlanBase() {}
  virtual void run() = 0;
};

template <typename T>
void dft1d(std::vector<std::complex<T> > &v, int sign) {
  const size_t n = v.size();
  if (n <= 1) return;
  const long double two_pi = 6.283185307179586476925286766559L;
  if ((n & (n - 1)) == 0) {
    /* bit-reversal permutation */
    for (size_t i = 1, j = 0; i < n; ++i) {
      size_t bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) std::swap(v[i], v[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
      const size_t half = len >> 1;
      for (size_t k = 0; k < half; ++k) {
        const long double ang = two_pi * (long double)k / (long double)len;
        const std::complex<T> w((T)std::cos(ang), (T)(sign * std::sin(ang)));
        for (size_t s = 0; s < n; s += len) {
          const std::complex<T> a = v[s + k];
          const std::complex<T> b = v[s + k + half] * w;
          v[s + k] = a + b;
          v[s + k + half] = a - b;
        }
      }
    }
    return;
  }
  std::vector<std::complex<T> > out(n);
  for (size_t k = 0; k < n; ++k) {
    std::complex<T> acc(0, 0);
    for (size_t j = 0; j < n; ++j) {
      const long double ang = two_pi * (long double)((k * j) % n) / (long double)n;
      acc += v[j] * std::complex<T>((T)std::cos(ang), (T)(sign * std::sin(ang)));
    }
    out[k] = acc;
  }
  v.swap(out);
}

/* Complex passes along dims 0 and 1 of an [n0][n1][m] complex array. */
template <typename T>
void passes01(std::complex<T> *a, int n0, int n1, int m, int sign) {
  std::vector<std::complex<T> > line;
  line.resize((size_t)n1);
  for (int i0 = 0; i0 < n0; ++i0)
    for (int k = 0; k < m; ++k) {
      for (int i1 = 0; i1 < n1; ++i1) line[(size_t)i1] = a[((size_t)i0 * n1 + i1) * m + k];
      dft1d(line, sign);
      for (int i1 = 0; i1 < n1; ++i1) a[((size_t)i0 * n1 + i1) * m + k] = line[(size_t)i1];
    }
  line.resize((size_t)n0);
  for (int i1 = 0; i1 < n1; ++i1)
    for (int k = 0; k < m; ++k) {
      for (int i0 = 0; i0 < n0; ++i0) line[(size_t)i0] = a[((size_t)i0 * n1 + i1) * m + k];
      dft1d(line, sign);
      for (int i0 = 0; i0 < n0; ++i0) a[((size_t)i0 * n1 + i1) * m + k] = line[(size_t)i0];
    }
}

template <typename T>
struct R2C : PlanBase {
  int n0, n1, n2;
  T *in;
  T (*out)[2];
  void run() {
    const int m = n2 / 2 + 1, pad = 2 * m;
    std::vector<std::complex<T> > work((size_t)n0 * n1 * m);
    std::vector<std::complex<T> > line((size_t)n2);
    for (int i0 = 0; i0 < n0; ++i0)
      for (int i1 = 0; i1 < n1; ++i1) {
        const T *row = in + ((size_t)i0 * n1 + i1) * pad;
        for (int j = 0; j < n2; ++j) line[(size_t)j] = std::complex<T>(row[j], 0);
        dft1d(line, -1);
        for (int k = 0; k < m; ++k) work[((size_t)i0 * n1 + i1) * m + k] = line[(size_t)k];
      }
    passes01(work.data(), n0, n1, m, -1);
    for (size_t i = 0; i < work.size(); ++i) {
      out[i][0] = work[i].real();
      out[i][1] = work[i].imag();
    }
  }
};

template <typename T>
struct C2R : PlanBase {
  int n0, n1, n2;
  T (*in)[2];
  T *out;
  void run() {
    const int m = n2 / 2 + 1, pad = 2 * m;
    std::vector<std::complex<T> > work((size_t)n0 * n1 * m);
    for (size_t i = 0; i < work.size(); ++i) work[i] = std::complex<T>(in[i][0], in[i][1]);
    passes01(work.data(), n0, n1, m, +1);
    std::vector<std::complex<T> > line((size_t)n2);
    for (int i0 = 0; i0 < n0; ++i0)
      for (int i1 = 0; i1 < n1; ++i1) {
        const std::complex<T> *h = &work[((size_t)i0 * n1 + i1) * m];
        for (int k = 0; k < n2; ++k)
          line[(size_t)k] = (k < m) ? h[k] : std::conj(h[n2 - k]);
        dft1d(line, +1);
        T *row = out + ((size_t)i0 * n1 + i1) * pad;
        for (int j = 0; j < n2; ++j) row[j] = line[(size_t)j].real();
      }
  }
};

} // namespace phn_fft_shim

#define PHN_FFTW_SHIM_API(PFX, T)                                                              \
  typedef phn_fft_shim::PlanBase *PFX##_plan;                                                  \
  inline void PFX##_mpi_init() {}                                                              \
  inline ptrdiff_t PFX##_mpi_local_size_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2h, int,      \
                                           ptrdiff_t *local_n0, ptrdiff_t *local_0_start) {    \
    *local_n0 = n0;                                                                            \
    *local_0_start = 0;                                                                        \
    return n0 * n1 * n2h;                                                                      \
  }                                                                                            \
  inline T *PFX##_alloc_real(size_t n) { return (T *)std::calloc(n, sizeof(T)); }              \
  inline PFX##_complex *PFX##_alloc_complex(size_t n) {                                        \
    return (PFX##_complex *)std::calloc(n, sizeof(PFX##_complex));                             \
  }                                                                                            \
  inline PFX##_plan PFX##_mpi_plan_dft_r2c_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, T *in, \
                                              PFX##_complex *out, int, unsigned) {             \
    phn_fft_shim::R2C<T> *p = new phn_fft_shim::R2C<T>();                                      \
    p->n0 = (int)n0; p->n1 = (int)n1; p->n2 = (int)n2; p->in = in; p->out = out;               \
    return p;                                                                                  \
  }                                                                                            \
  inline PFX##_plan PFX##_mpi_plan_dft_c2r_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2,        \
                                              PFX##_complex *in, T *out, int, unsigned) {      \
    phn_fft_shim::C2R<T> *p = new phn_fft_shim::C2R<T>();                                      \
    p->n0 = (int)n0; p->n1 = (int)n1; p->n2 = (int)n2; p->in = in; p->out = out;               \
    return p;                                                                                  \
  }                                                                                            \
  inline void PFX##_execute(PFX##_plan p) { p->run(); }                                        \
  inline void PFX##_destroy_plan(PFX##_plan p) { delete p; }

PHN_FFTW_SHIM_API(fftw, double)
PHN_FFTW_SHIM_API(fftwf, float)
PHN_FFTW_SHIM_API(fftwl, long double)

#endif
