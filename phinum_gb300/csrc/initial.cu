// Initial conditions on the GPU: SetInitialConditions for `initialize` 0-4,
// with or without charge, static or expanding box (initialconditions.cpp:
// 45-723, clusterfft.cpp:55-182), with the reference's own random stream.  The
// expanding box (:459-465, :504-510, :581-583, :656-658) seeds the
// scale-invariant occupation 2 pi^2 2.1e-9 phi0_0^2 omega_p / p^3 below QS,
// uses Omega^2 = p^2 + (1 + 2 H_0 T0) M^2, E = H_0 A, and adds phi0_0 H_0 to
// the first momentum component.
//
// The reference draws from drand48 (seeded by srand48, initialconditions.cpp:
// 14-22) in mode order (pz, px, py <= N/2, component): per mode two phases
// (two draws), then two Gaussians from one polar Box-Muller acceptance
// (Gauss(), :27-41: pairs of draws until the point falls inside the unit
// disc; the second Gaussian of the pair is cached for the next call).  Every
// mode consumes 2 + 2k draws, so every mode starts on an even draw and the
// stream splits into pairs: one phase pair, then trial pairs up to the first
// accepted one.  Which pair belongs to which mode is a two-state automaton
// over the acceptance flags ("next pair is a phase pair" / "a trial pair");
// it is evaluated with a parallel prefix over chunks of pairs.
//
// The charged variant with Nc = 2 (withcharge 1, :132-147) draws one phase
// and one Gaussian per mode (component 1; component 0 reuses the draws of the
// two modes before).  Its stream is u_0, then trials up to an accepted pair
// (whose two Gaussians serve two modes), then u_1 u_2, trials, u_3 u_4, ...:
// one draw later, the same automaton over pairs, entered in the trial state.
//
//   ic_pairs    drand48 by jump-ahead (X <- A^k X + C_k mod 2^48): each thread
//               one chunk of pairs; stores the pairs (exact doubles X / 2^48),
//               and the chunk's automaton transition for both entry states
//   ic_scan_*   prefix over chunks: per block in shared memory, then over
//               blocks on one thread, then the entry state and first mode of
//               every chunk
//   ic_assign   each chunk re-walks its pairs and records, per mode, the phase
//               pair and the accepted pair
//   ic_modes    amplitudes in FP64 with the reference's expressions and order
//               (occupation, Omega, F1, F2, A = F1/sqrt(Omega), E = F2 sqrt(Omega))
//   ic_reality  ensureRealResult (clusterfft.cpp:55-139) on the py = 0 and
//               py = N/2 planes: the mode visited first sets its partner
//   cuFFT Z2D   fftPtoX (clusterfft.cpp:148-182): the complex array is
//               [pz][px][py], so lattice y is the halved axis
//   ic_store    X / L^3 * sqrt(L^3) + phi0 into the handle's [z][y][x] fields
//               (a shared-memory transpose of x and y)
//
// The stream, the acceptance decisions and the mode assignment are exact, and
// the per-axis momenta are the C library's values (computed on the host); the
// Box-Muller log and the phases' cos/sin are CUDA's, which may differ from the
// C library's in the last bit, and cuFFT rounds differently from FFTW.
#include <cufft.h>
#include <math.h>
#include <string.h>

#include "phn_internal.h"

namespace phn {

constexpr unsigned long long LCG_A = 0x5DEECE66DULL, LCG_C = 0xBULL, LCG_MASK = (1ULL << 48) - 1;
constexpr int IC_CHUNK = 64;     // pairs per thread in ic_pairs / ic_assign
constexpr int IC_THREADS = 256;  // chunks per scan block

struct Lcg {  // X -> a X + c (mod 2^48)
  unsigned long long a, c;
};

__host__ __device__ inline Lcg lcg_then(Lcg f, Lcg g) {  // f first, then g
  Lcg h;
  h.a = (g.a * f.a) & LCG_MASK;
  h.c = (g.a * f.c + g.c) & LCG_MASK;
  return h;
}

// k steps of the drand48 recurrence
__host__ __device__ inline Lcg lcg_pow(unsigned long long k) {
  Lcg r = {1, 0}, b = {LCG_A, LCG_C};
  while (k) {
    if (k & 1) r = lcg_then(r, b);
    b = lcg_then(b, b);
    k >>= 1;
  }
  return r;
}

// Automaton over pairs: state 0 = the next pair is a mode's phase pair,
// state 1 = the next pair is a Box-Muller trial.  A transition records, for
// each entry state, the exit state and the number of modes completed.
struct Trans {
  unsigned char e[2];
  unsigned int n[2];
};

__device__ __forceinline__ Trans trans_id() {
  Trans t;
  t.e[0] = 0;
  t.e[1] = 1;
  t.n[0] = t.n[1] = 0;
  return t;
}

__device__ __forceinline__ Trans trans_then(const Trans &f, const Trans &g) {  // f first
  Trans h;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    h.e[s] = g.e[f.e[s]];
    h.n[s] = f.n[s] + g.n[f.e[s]];
  }
  return h;
}

// The reference's acceptance test (initialconditions.cpp:33-35) in IEEE
// operations without contraction: x = 2u - 1, y = 2v - 1, sqrt(x^2 + y^2) < 1.
__device__ __forceinline__ bool accepted(double u, double v) {
  const double x = __dsub_rn(__dmul_rn(2.0, u), 1.0), y = __dsub_rn(__dmul_rn(2.0, v), 1.0);
  const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
  return r < 1.0;
}

// Stream pairs [chunk * IC_CHUNK, ...) of the drand48 stream that starts in
// state x0 (srand48); draw k is X_{k+1} / 2^48.
__global__ void ic_pairs(unsigned long long x0, long long npairs, double2 *__restrict__ uv, Trans *__restrict__ trans,
                         long long nchunks) {
  const long long chunk = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (chunk >= nchunks) return;
  const long long p0 = chunk * IC_CHUNK;
  const Lcg jump = lcg_pow(2ULL * (unsigned long long)p0);
  unsigned long long x = (jump.a * x0 + jump.c) & LCG_MASK;
  Trans t = trans_id();
  const long long p1 = min(p0 + IC_CHUNK, npairs);
  for (long long p = p0; p < p1; ++p) {
    x = (LCG_A * x + LCG_C) & LCG_MASK;
    const double u = (double)x * 0x1p-48;
    x = (LCG_A * x + LCG_C) & LCG_MASK;
    const double v = (double)x * 0x1p-48;
    uv[p] = make_double2(u, v);
    const bool acc = accepted(u, v);
    // one pair: state 0 -> 1; state 1 -> 0 with a mode completed if accepted
    Trans step;
    step.e[0] = 1;
    step.n[0] = 0;
    step.e[1] = acc ? 0 : 1;
    step.n[1] = acc ? 1 : 0;
    t = trans_then(t, step);
  }
  trans[chunk] = t;
}

// Exclusive prefix of the chunk transitions inside each block (shared-memory
// Hillis-Steele scan) and the block's total.
__global__ void ic_scan_blocks(const Trans *__restrict__ trans, long long nchunks, Trans *__restrict__ excl,
                               Trans *__restrict__ block_total) {
  __shared__ Trans sh[2][IC_THREADS];
  const long long i = blockIdx.x * (long long)IC_THREADS + threadIdx.x;
  Trans mine = i < nchunks ? trans[i] : trans_id();
  int cur = 0;
  sh[cur][threadIdx.x] = mine;
  __syncthreads();
  for (int off = 1; off < IC_THREADS; off <<= 1) {
    Trans v = sh[cur][threadIdx.x];
    if (threadIdx.x >= off) v = trans_then(sh[cur][threadIdx.x - off], v);
    sh[1 - cur][threadIdx.x] = v;
    cur = 1 - cur;
    __syncthreads();
  }
  // sh[cur] holds inclusive prefixes
  if (i < nchunks) excl[i] = threadIdx.x == 0 ? trans_id() : sh[cur][threadIdx.x - 1];
  if (threadIdx.x == IC_THREADS - 1) block_total[blockIdx.x] = sh[cur][threadIdx.x];
}

// Entry state and modes completed before each block, from the start state
// (0: a phase pair first; 1: a trial first, the charged stream).
__global__ void ic_scan_top(const Trans *__restrict__ block_total, long long nblocks, int start,
                            unsigned char *__restrict__ bstate, unsigned long long *__restrict__ bmodes) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  unsigned char s = (unsigned char)start;
  unsigned long long n = 0;
  for (long long b = 0; b < nblocks; ++b) {
    bstate[b] = s;
    bmodes[b] = n;
    const Trans &t = block_total[b];
    n += t.n[s];
    s = t.e[s];
  }
  bstate[nblocks] = s;
  bmodes[nblocks] = n;
}

// Each chunk re-walks its pairs from its entry state and records, for every
// mode it touches, the phase pair and the accepted pair.
__global__ void ic_assign(const double2 *__restrict__ uv, long long npairs, long long nchunks,
                          const Trans *__restrict__ excl, const unsigned char *__restrict__ bstate,
                          const unsigned long long *__restrict__ bmodes, long long nmodes,
                          long long *__restrict__ phase_pair, long long *__restrict__ acc_pair) {
  const long long chunk = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (chunk >= nchunks) return;
  const long long b = chunk / IC_THREADS;
  const Trans &pre = excl[chunk];
  const unsigned char sb = bstate[b];
  int s = pre.e[sb];
  unsigned long long m = bmodes[b] + pre.n[sb];
  const long long p0 = chunk * IC_CHUNK, p1 = min(p0 + IC_CHUNK, npairs);
  for (long long p = p0; p < p1 && (long long)m < nmodes; ++p) {
    if (s == 0) {
      phase_pair[m] = p;
      s = 1;
    } else {
      const double2 w = uv[p];
      if (accepted(w.x, w.y)) {
        acc_pair[m] = p;
        ++m;
        s = 0;
      }
    }
  }
}

struct IcConsts {
  int N, Nc, justnoise, expansion;
  int initialize, withcharge;
  double a, QS, scale2, amplitude, noise, m2_long, m2_trans;
  double H0;
  double a0sq;      // 1. + 2.*H_0*T0: the initial scale factor squared
  double spectrum;  // 2.*acos(-1.)*acos(-1.)*2.1e-9*phi0_0*phi0_0
  // initialize 0-2 and 4 (host values in the reference's order)
  double abs_m;     // fabs(M_sqr)
  double w_long, w_trans;  // 3.*sqr(Temperature)*sqr(phi0)/(6.*Nc), sqr(T)*sqr(phi0)/(6.*Nc) (init 0);
                           // 3.*sqr(phi0)/(6.*Nc), sqr(phi0)/(6.*Nc) (init 1, 2)
  double occ0;      // FAmp*Lambda (init 0)
  double chi2;      // sqr(chi) (init 1)
  double two_qs;    // 2.0*QS (init 1)
  double temperature;
  double u0;        // the charged stream's first draw
};

// Per-axis lattice momentum as initialconditions.cpp:88-113 writes it,
// evaluated on the host with the C library's sin (the reference's values).
static double ic_p_host(int n, int N, double a) {
  if (n < N / 2 + 1) return 2.0 / (a) * sin(n * acos(-1.) / N);
  return -2.0 / (a) * sin(n * acos(-1.) / N);
}

// The chopped plateau of initialize 2-4: Noise below scale2 (everywhere
// when scale2 == 0), else 0.
__device__ __forceinline__ double ic_plateau(const IcConsts &k, double root) {
  return k.scale2 == 0 ? k.noise : (root < k.scale2 ? k.noise : 0.0);
}

// Occupation and Omega of one mode and component, each `initialize` branch
// with its own comparisons (initialconditions.cpp:163-257 with charge,
// :308-556 without); IEEE operations in the reference's order.
__device__ void ic_occ_omega(const IcConsts &k, int a, double pt, double nu, double psqr, double *occ,
                             double *omega) {
  const double m2 = a == 0 ? k.m2_long : k.m2_trans;
  switch (k.initialize) {
    case 0:
      *omega = __dsqrt_rn(__dsub_rn(__dadd_rn(psqr, k.abs_m), a == 0 ? k.w_long : k.w_trans));
      *occ = k.occ0;
      return;
    case 1: {
      const double pchisqr = __dadd_rn(__dmul_rn(pt, pt), __dmul_rn(k.chi2, __dmul_rn(nu, nu)));
      const double root = __dsqrt_rn(pchisqr);
      *occ = root < k.QS ? k.amplitude : (root < k.two_qs ? k.noise : 0.0);
      *omega = __dsqrt_rn(__dsub_rn(__dadd_rn(psqr, k.abs_m), a == 0 ? k.w_long : k.w_trans));
      return;
    }
    case 2: {
      const double root = __dsqrt_rn(psqr);  // pchisqr = sqr(pt)+sqr(nu) = psqr
      *occ = (k.justnoise == 0 && root < k.QS) ? __dadd_rn(k.amplitude, k.noise) : ic_plateau(k, root);
      *omega = __dsqrt_rn(__dsub_rn(__dadd_rn(psqr, k.abs_m), a == 0 ? k.w_long : k.w_trans));
      return;
    }
    case 3: {
      const double root = __dsqrt_rn(psqr);
      if (k.withcharge) {  // :255-291, static forms
        *occ = (k.justnoise == 0 && root < k.QS) ? __dadd_rn(k.amplitude, k.noise) : ic_plateau(k, root);
        *omega = __dsqrt_rn(__dadd_rn(psqr, m2));
        return;
      }
      if (k.expansion) {  // :459-465, :504-510
        if (k.justnoise == 0 && psqr > 0. && psqr < __dmul_rn(k.QS, k.QS)) {
          const double omegap = __dsqrt_rn(__dadd_rn(psqr, __dmul_rn(k.a0sq, k.m2_long)));
          *occ = __dmul_rn(__ddiv_rn(__ddiv_rn(k.spectrum, psqr), __dsqrt_rn(psqr)), omegap);
        } else {
          *occ = ic_plateau(k, root);
        }
        *omega = __dsqrt_rn(__dadd_rn(psqr, __dmul_rn(k.a0sq, m2)));
      } else {
        *occ = (k.justnoise == 0 && psqr < __dmul_rn(k.QS, k.QS)) ? __dadd_rn(k.amplitude, k.noise)
                                                                   : ic_plateau(k, root);
        *omega = __dsqrt_rn(__dadd_rn(psqr, m2));
      }
      return;
    }
    default: {  // 4 (:514-556)
      const double root = __dsqrt_rn(psqr);
      *occ = (k.justnoise == 0 && psqr < __dmul_rn(k.QS, k.QS))
                 ? __dadd_rn(__ddiv_rn(k.temperature, __dsqrt_rn(__dadd_rn(psqr, k.m2_long))), k.noise)
                 : ic_plateau(k, root);
      *omega = __dsqrt_rn(__dadd_rn(psqr, m2));
      return;
    }
  }
}

// Box-Muller of an accepted pair (initialconditions.cpp:36-39): gauss1 and
// the cached gauss2.
__device__ __forceinline__ void ic_box_muller(double2 g, double *g1, double *g2) {
  const double x = __dsub_rn(__dmul_rn(2.0, g.x), 1.0), y = __dsub_rn(__dmul_rn(2.0, g.y), 1.0);
  const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
  const double c = __ddiv_rn(x, r), s = __ddiv_rn(y, r);
  *g1 = __dmul_rn(c, __dsqrt_rn(__dmul_rn(-2.0, log(__dmul_rn(r, r)))));
  *g2 = __dmul_rn(__ddiv_rn(s, c), *g1);
}

// A and E of one mode and component from its phases and |Gaussians|
// (initialconditions.cpp:563-587): F = sqrt(occ) g (cos th, sin th),
// A = F1 / sqrt(Omega), E = F2 sqrt(Omega), or E = A H_0 in the expanding
// box without charge; both 0 where |Omega| < 1e-8.
__device__ void ic_amplitudes(const IcConsts &k, int a, int pz, int px, int py, const double *__restrict__ ptab,
                              double phase1, double phase2, double gauss1, double gauss2, double2 *fa_out,
                              double2 *fe_out) {
  const double nu = pz == 0 ? 0.0 : ptab[pz];
  const double ppx = ptab[px];
  const double ppy = ptab[py];  // py <= N/2: the positive branch
  const double pt = __dsqrt_rn(__dadd_rn(__dmul_rn(ppx, ppx), __dmul_rn(ppy, ppy)));
  const double psqr = __dadd_rn(__dmul_rn(pt, pt), __dmul_rn(nu, nu));
  double occ, omega;
  ic_occ_omega(k, a, pt, nu, psqr, &occ, &omega);
  const double amp1 = __dmul_rn(__dsqrt_rn(occ), gauss1), amp2 = __dmul_rn(__dsqrt_rn(occ), gauss2);
  double2 fa = make_double2(0.0, 0.0), fe = make_double2(0.0, 0.0);
  if (!(fabs(omega) < 1e-8)) {
    const double so = __dsqrt_rn(omega);
    fa = make_double2(__ddiv_rn(__dmul_rn(amp1, cos(phase1)), so), __ddiv_rn(__dmul_rn(amp1, sin(phase1)), so));
    if (k.expansion && !k.withcharge)  // EFieldP = AFieldP * H_0 (:581-583)
      fe = make_double2(__dmul_rn(fa.x, k.H0), __dmul_rn(fa.y, k.H0));
    else
      fe = make_double2(__dmul_rn(__dmul_rn(amp2, cos(phase2)), so), __dmul_rn(__dmul_rn(amp2, sin(phase2)), so));
  }
  *fa_out = fa;
  *fe_out = fe;
}

// One (mode, component) of the uncharged stream (and the charged one for
// Nc != 2, which draws alike): two phases from its phase pair, two
// Gaussians from its accepted pair.  A and E are [a][pz][px][py] complex
// arrays.
__global__ void ic_modes(const IcConsts k, const double *__restrict__ ptab, const double2 *__restrict__ uv,
                         const long long *__restrict__ phase_pair,
                         const long long *__restrict__ acc_pair, long long nmodes, double2 *__restrict__ A,
                         double2 *__restrict__ E) {
  const long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (m >= nmodes) return;
  const int N = k.N, M = N / 2 + 1;
  const int a = (int)(m % k.Nc);
  const long long pos = m / k.Nc;  // py + px M + pz N M: the mode loop order
  const int py = (int)(pos % M), px = (int)((pos / M) % N), pz = (int)(pos / ((long long)M * N));
  // phases and Gaussians (initialconditions.cpp:27-41, 344-349)
  const double2 ph = uv[phase_pair[m]];
  const double two_pi = __dmul_rn(2.0, acos(-1.));
  double g1, g2;
  ic_box_muller(uv[acc_pair[m]], &g1, &g2);
  double2 fa, fe;
  ic_amplitudes(k, a, pz, px, py, ptab, __dmul_rn(two_pi, ph.x), __dmul_rn(two_pi, ph.y), fabs(g1), fabs(g2), &fa,
                &fe);
  const size_t o = (size_t)a * N * N * M + ((size_t)pz * N + px) * M + py;
  A[o] = fa;
  E[o] = fe;
}

// The charged stream with Nc = 2: mode m's draw u_m (u_0 the first draw;
// then u_{2j-1}, u_{2j} the j-th phase pair) and |Gaussian| (the first or
// the cached second value of accepted pair m/2).  Component 1 of mode m
// takes (u_m, u_{m-1}) and (g_m, g_{m-1}); component 0 those of m-1 and m-2;
// values before the stream began are the reference's uninitialized locals,
// read as 0 (as its pinned build reads them).
__device__ __forceinline__ double ic_q_phase(const IcConsts &k, const double2 *__restrict__ uv,
                                             const long long *__restrict__ phase_pair, long long m) {
  if (m < 0) return 0.0;
  const double u = m == 0 ? k.u0 : ((m & 1) ? uv[phase_pair[(m + 1) / 2]].x : uv[phase_pair[m / 2]].y);
  return __dmul_rn(__dmul_rn(2.0, acos(-1.)), u);
}

__device__ __forceinline__ double ic_q_gauss(const double2 *__restrict__ uv, const long long *__restrict__ acc_pair,
                                             long long m) {
  if (m < 0) return 0.0;
  double g1, g2;
  ic_box_muller(uv[acc_pair[m / 2]], &g1, &g2);
  return fabs((m & 1) ? g2 : g1);
}

__global__ void ic_modes_q(const IcConsts k, const double *__restrict__ ptab, const double2 *__restrict__ uv,
                           const long long *__restrict__ phase_pair, const long long *__restrict__ acc_pair,
                           long long nmodes, double2 *__restrict__ A, double2 *__restrict__ E) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nmodes) return;
  const int N = k.N, M = N / 2 + 1;
  const int a = (int)(t & 1);
  const long long pos = t >> 1;
  const int py = (int)(pos % M), px = (int)((pos / M) % N), pz = (int)(pos / ((long long)M * N));
  const long long m = a == 1 ? pos : pos - 1;
  double2 fa, fe;
  ic_amplitudes(k, a, pz, px, py, ptab, ic_q_phase(k, uv, phase_pair, m), ic_q_phase(k, uv, phase_pair, m - 1),
                ic_q_gauss(uv, acc_pair, m), ic_q_gauss(uv, acc_pair, m - 1), &fa, &fe);
  const size_t o = (size_t)a * N * N * M + ((size_t)pz * N + px) * M + py;
  A[o] = fa;
  E[o] = fe;
}

// ensureRealResult on the py = 0 and py = N/2 planes (clusterfft.cpp:55-139):
// the mode visited first in (pz, px) order sets its partner to its
// conjugate; a self-conjugate mode becomes |F| sgn(Re F) (sgn(0) = -1,
// clusterfft.cpp:10-16).
__global__ void ic_reality(double2 *__restrict__ F, int N, int Nc) {
  const int M = N / 2 + 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long per = 2LL * N * N;
  if (t >= per * Nc) return;
  const int a = (int)(t / per);
  const long long r = t % per;
  const int py = (r / ((long long)N * N)) == 0 ? 0 : N / 2;
  const int pz = (int)((r / N) % N), px = (int)(r % N);
  const int mpz = (N - pz) % N, mpx = (N - px) % N;
  double2 *base = F + (size_t)a * N * N * M;
  const size_t i = ((size_t)pz * N + px) * M + py;
  if (pz == mpz && px == mpx) {
    const double2 v = base[i];
    const double mag = hypot(v.x, v.y);
    base[i] = make_double2(v.x > 0 ? mag : -mag, 0.0);
  } else if (pz < mpz || (pz == mpz && px < mpx)) {
    const double2 v = base[i];
    base[((size_t)mpz * N + mpx) * M + py] = make_double2(v.x, -v.y);
  }
}

// out[z][y][x] = (X[z][x][y] * scale + offset) + offset2: 32 x 32 tiles
// through shared memory.
template <typename T>
__global__ void ic_store(const double *__restrict__ X, T *__restrict__ out, int N, double scale, double offset,
                         double offset2) {
  __shared__ double tile[32][33];
  const int z = blockIdx.z;
  const int x0 = blockIdx.y * 32, y0 = blockIdx.x * 32;
  const size_t plane = (size_t)z * N * N;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int x = x0 + j, y = y0 + threadIdx.x;
    if (x < N && y < N) tile[j][threadIdx.x] = X[plane + (size_t)x * N + y];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int y = y0 + j, x = x0 + threadIdx.x;
    if (x < N && y < N) out[plane + (size_t)y * N + x] = (T)((tile[threadIdx.x][j] * scale + offset) + offset2);
  }
}

}  // namespace phn

using namespace phn;

extern "C" {

static int run_initial_conditions(phn_handle *h, const phn_ic_params *ic, const phn_ic_mode *md) {
  if (!h || !ic || !md) return set_error(PHN_ERR_INVALID, "NULL argument");
  const int N = h->p.N, Nc = h->p.Nc;
  if (N % 2 != 0) return set_error(PHN_ERR_UNSUPPORTED, "initial conditions need an even N");
  if (md->init_mode < 0 || md->init_mode > 4) return set_error(PHN_ERR_INVALID, "initialize %d", md->init_mode);
  if (md->charged != 0 && md->charged != 1) return set_error(PHN_ERR_INVALID, "withcharge %d", md->charged);
  if (md->init_mode == 4 && md->charged)
    return set_error(PHN_ERR_UNSUPPORTED, "initialize 4 has no charged form (the reference sets no occupation)");
  const int M = N / 2 + 1;
  // the charged stream with Nc = 2: one accepted pair per two modes; the
  // automaton runs one mode further for the last modes' phases
  const bool paired = md->charged && Nc == 2;
  const long long nspatial = (long long)N * N * M;
  const long long nmodes = paired ? nspatial / 2 + 1 : nspatial * Nc;
  const long long nthreads = paired ? nspatial * 2 : nmodes;
  // pairs: one phase pair per mode plus 4/pi trials on average; 2.5 per mode
  // leaves a margin of thousands of standard deviations
  const long long npairs = nmodes * 5 / 2 + 65536;
  const long long nchunks = (npairs + IC_CHUNK - 1) / IC_CHUNK;
  const long long nsblocks = (nchunks + IC_THREADS - 1) / IC_THREADS;
  const size_t nspec = (size_t)N * N * M;
  cudaStream_t st = h->stream;
  double2 *uv = nullptr, *A = nullptr, *E = nullptr;
  Trans *trans = nullptr, *excl = nullptr, *btot = nullptr;
  unsigned char *bstate = nullptr;
  unsigned long long *bmodes = nullptr;
  long long *phase_pair = nullptr, *acc_pair = nullptr;
  double *X = nullptr, *ptab = nullptr;
  unsigned long long done = 0;
  cufftHandle plan = 0;
  bool plan_ok = false;
  int r = PHN_OK;
  cudaError_t e = cudaSuccess;
#define ICK(call)                          \
  do {                                     \
    e = (call);                            \
    if (e != cudaSuccess) {                \
      r = cuda_error(e, #call);            \
      goto cleanup;                        \
    }                                      \
  } while (0)
  {
    ICK(cudaMalloc(&uv, npairs * sizeof(double2)));
    ICK(cudaMalloc(&trans, nchunks * sizeof(Trans)));
    ICK(cudaMalloc(&excl, nchunks * sizeof(Trans)));
    ICK(cudaMalloc(&btot, nsblocks * sizeof(Trans)));
    ICK(cudaMalloc(&bstate, (nsblocks + 1) * sizeof(unsigned char)));
    ICK(cudaMalloc(&bmodes, (nsblocks + 1) * sizeof(unsigned long long)));
    ICK(cudaMalloc(&phase_pair, nmodes * sizeof(long long)));
    ICK(cudaMalloc(&acc_pair, nmodes * sizeof(long long)));
    ICK(cudaMalloc(&A, (size_t)Nc * nspec * sizeof(double2)));
    ICK(cudaMalloc(&E, (size_t)Nc * nspec * sizeof(double2)));
    ICK(cudaMalloc(&X, (size_t)N * N * N * sizeof(double)));
    ICK(cudaMalloc(&ptab, N * sizeof(double)));
    {
      double tab[4096];
      if (N > 4096) {
        r = set_error(PHN_ERR_UNSUPPORTED, "N > 4096");
        goto cleanup;
      }
      for (int n = 0; n < N; ++n) tab[n] = ic_p_host(n, N, h->p.a);
      ICK(cudaMemcpy(ptab, tab, N * sizeof(double), cudaMemcpyHostToDevice));
    }
    // srand48(seed): X0 = (seed mod 2^32) 2^16 + 0x330E; the charged
    // stream's pairs start after its first draw
    unsigned long long x0 = (((unsigned long long)ic->seed & 0xFFFFFFFFULL) << 16) | 0x330EULL;
    double u0 = 0.0;
    if (paired) {
      x0 = (LCG_A * x0 + LCG_C) & LCG_MASK;
      u0 = (double)x0 * 0x1p-48;
    }
    const int tb = 128;
    ic_pairs<<<(unsigned)((nchunks + tb - 1) / tb), tb, 0, st>>>(x0, npairs, uv, trans, nchunks);
    ICK(cudaGetLastError());
    ic_scan_blocks<<<(unsigned)nsblocks, IC_THREADS, 0, st>>>(trans, nchunks, excl, btot);
    ICK(cudaGetLastError());
    ic_scan_top<<<1, 1, 0, st>>>(btot, nsblocks, paired ? 1 : 0, bstate, bmodes);
    ICK(cudaGetLastError());
    ICK(cudaMemcpyAsync(&done, bmodes + nsblocks, sizeof(done), cudaMemcpyDeviceToHost, st));
    ICK(cudaStreamSynchronize(st));
    if ((long long)done < nmodes) {
      r = set_error(PHN_ERR_INVALID, "random stream too short (%llu of %lld modes)", done, nmodes);
      goto cleanup;
    }
    ICK(cudaMemsetAsync(phase_pair, 0, nmodes * sizeof(long long), st));
    ic_assign<<<(unsigned)((nchunks + tb - 1) / tb), tb, 0, st>>>(uv, npairs, nchunks, excl, bstate, bmodes, nmodes,
                                                                  phase_pair, acc_pair);
    ICK(cudaGetLastError());
    IcConsts k;
    k.N = N;
    k.Nc = Nc;
    k.justnoise = ic->justnoise;
    k.a = h->p.a;
    k.QS = ic->QS;
    k.scale2 = ic->scale2;
    k.amplitude = ic->amplitude;
    k.noise = ic->noise;
    k.m2_long = ic->m2_long;
    k.m2_trans = ic->m2_trans;
    k.expansion = h->p.expanding;
    k.H0 = h->p.H0;
    k.a0sq = 1. + 2. * h->p.H0 * h->p.T0;
    k.spectrum = 2. * acos(-1.) * acos(-1.) * 2.1e-9 * ic->phi0[0] * ic->phi0[0];
    k.initialize = md->init_mode;
    k.withcharge = md->charged;
    k.abs_m = fabs(h->p.m_sqr);
    // the mode-independent parts of Omega and the occupation, in the
    // reference's order (initialconditions.cpp:166-171, :198-203, :245-248)
    if (md->init_mode == 0) {
      k.w_long = 3. * (md->temperature * md->temperature) * (md->phi0 * md->phi0) / (6. * Nc);
      k.w_trans = (md->temperature * md->temperature) * (md->phi0 * md->phi0) / (6. * Nc);
    } else {
      k.w_long = 3. * (md->phi0 * md->phi0) / (6. * Nc);
      k.w_trans = (md->phi0 * md->phi0) / (6. * Nc);
    }
    k.occ0 = md->famp * md->lambda;
    k.chi2 = md->chi * md->chi;
    k.two_qs = 2.0 * ic->QS;
    k.temperature = md->temperature;
    k.u0 = u0;
    if (paired)
      ic_modes_q<<<(unsigned)((nthreads + 255) / 256), 256, 0, st>>>(k, ptab, uv, phase_pair, acc_pair, nthreads, A,
                                                                     E);
    else
      ic_modes<<<(unsigned)((nthreads + 255) / 256), 256, 0, st>>>(k, ptab, uv, phase_pair, acc_pair, nthreads, A,
                                                                   E);
    ICK(cudaGetLastError());
    const long long nre = 2LL * N * N * Nc;
    ic_reality<<<(unsigned)((nre + 255) / 256), 256, 0, st>>>(A, N, Nc);
    ic_reality<<<(unsigned)((nre + 255) / 256), 256, 0, st>>>(E, N, Nc);
    ICK(cudaGetLastError());
    h->launches += 8;
    if (cufftPlan3d(&plan, N, N, N, CUFFT_Z2D) != CUFFT_SUCCESS) {
      r = set_error(PHN_ERR_CUDA, "cufftPlan3d (Z2D %d^3) failed", N);
      goto cleanup;
    }
    plan_ok = true;
    if (cufftSetStream(plan, st) != CUFFT_SUCCESS) {
      r = set_error(PHN_ERR_CUDA, "cufftSetStream failed");
      goto cleanup;
    }
    // fftPtoX divides by L^3 (clusterfft.cpp:150,179), the caller multiplies
    // by sqrt(L^3) (initialconditions.cpp:638)
    const double L = h->p.a * N;
    const double norm = (L * L) * (N * h->p.a);
    const double scale = sqrt(norm) / norm;
    const double phi0[2] = {ic->phi0[0], ic->phi0[1]}, pi0[2] = {ic->pi0[0], ic->pi0[1]};
    const dim3 sg((N + 31) / 32, (N + 31) / 32, N), sb(32, 8);
    for (int f = 0; f < 2; ++f)
      for (int a = 0; a < Nc; ++a) {
        double2 *src = (f == 0 ? A : E) + (size_t)a * nspec;
        if (cufftExecZ2D(plan, (cufftDoubleComplex *)src, X) != CUFFT_SUCCESS) {
          r = set_error(PHN_ERR_CUDA, "cufftExecZ2D failed");
          goto cleanup;
        }
        // initialize 3 and 4 add phi0_0/1, pi0_0/1 (and the expanding box's
        // Pi_0 += phi0_0 H_0, initialconditions.cpp:657), the others phi0,
        // pi0 to component 0 only (:673-686)
        const bool own = md->init_mode == 3 || md->init_mode == 4;
        const double off = own ? (a < 2 ? (f == 0 ? phi0[a] : pi0[a]) : 0.0)
                               : (a == 0 ? (f == 0 ? md->phi0 : md->pi0) : 0.0);
        const double off2 = (own && h->p.expanding && f == 1 && a == 0) ? phi0[0] * h->p.H0 : 0.0;
        void *dst = f == 0 ? h->phi[h->cur] : h->pi;
        if (h->p.precision == PHN_FP64) {
          ic_store<double><<<sg, sb, 0, st>>>(X, (double *)dst + (size_t)a * h->V, N, scale, off, off2);
        } else {
          ic_store<float><<<sg, sb, 0, st>>>(X, (float *)dst + (size_t)a * h->V, N, scale, off, off2);
        }
        ICK(cudaGetLastError());
        h->launches++;
      }
    if (h->p.precision == PHN_FP32_KAHAN) {
      ICK(cudaMemsetAsync(h->cphi, 0, h->V * h->p.Nc * sizeof(float), st));
      ICK(cudaMemsetAsync(h->cpi, 0, h->V * h->p.Nc * sizeof(float), st));
    }
    ICK(cudaStreamSynchronize(st));
  }
cleanup:
#undef ICK
  if (plan_ok) cufftDestroy(plan);
  cudaFree(uv);
  cudaFree(trans);
  cudaFree(excl);
  cudaFree(btot);
  cudaFree(bstate);
  cudaFree(bmodes);
  cudaFree(phase_pair);
  cudaFree(acc_pair);
  cudaFree(A);
  cudaFree(E);
  cudaFree(X);
  cudaFree(ptab);
  return r;
}

int phn_initial_conditions(phn_handle *h, const phn_ic_params *ic) {
  phn_ic_mode md;
  memset(&md, 0, sizeof(md));
  md.init_mode = 3;
  return run_initial_conditions(h, ic, &md);
}

int phn_initial_conditions_mode(phn_handle *h, const phn_ic_params *ic, const phn_ic_mode *mode) {
  return run_initial_conditions(h, ic, mode);
}

}  // extern "C"
