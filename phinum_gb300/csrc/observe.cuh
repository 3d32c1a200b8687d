// Observation accumulators shared by the lattice kernels: per-site terms of
// CalculateVolumeAverages + CalculateExtrema (fieldanalysis.cpp:319-699) and
// the deterministic warp/block reduction into per-block FP64 records.
#pragma once

#include <math.h>

#include "phn_internal.h"

namespace phn {

// ----------------------------------------------------------- accumulators
struct Acc {
  double s[NSUM];
  double minv, maxv, absv;
  long long mini, maxi, absi;
  __device__ void init() {
#pragma unroll
    for (int j = 0; j < NSUM; ++j) s[j] = 0.0;
    // CalculateExtrema's starting values (fieldanalysis.cpp:324-325)
    minv = 10000000.0;
    maxv = -10000000.0;
    absv = 0.0;
    mini = maxi = absi = LLONG_MAX;
  }
  // Strict comparisons as in the reference; equal values keep the smaller
  // index, which is the first one the reference's linear scan meets.
  __device__ void take_max(double v, long long i) {
    if (v > maxv || (v == maxv && i < maxi && v > -10000000.0)) { maxv = v; maxi = i; }
  }
  __device__ void take_min(double v, long long i) {
    if (v < minv || (v == minv && i < mini && v < 10000000.0)) { minv = v; mini = i; }
  }
  __device__ void take_abs(double v, long long i) {
    if (v > absv || (v == absv && i < absi && v > 0.0)) { absv = v; absi = i; }
  }
};

__device__ __forceinline__ void combine(Acc &a, const Acc &b) {
#pragma unroll
  for (int j = 0; j < NSUM; ++j) a.s[j] += b.s[j];
  if (b.maxi != LLONG_MAX) a.take_max(b.maxv, b.maxi);
  if (b.mini != LLONG_MAX) a.take_min(b.minv, b.mini);
  if (b.absi != LLONG_MAX) a.take_abs(b.absv, b.absi);
}

__device__ __forceinline__ Acc shfl_down(const Acc &a, int off) {
  Acc b;
#pragma unroll
  for (int j = 0; j < NSUM; ++j) b.s[j] = __shfl_down_sync(0xffffffffu, a.s[j], off);
  b.minv = __shfl_down_sync(0xffffffffu, a.minv, off);
  b.maxv = __shfl_down_sync(0xffffffffu, a.maxv, off);
  b.absv = __shfl_down_sync(0xffffffffu, a.absv, off);
  b.mini = __shfl_down_sync(0xffffffffu, a.mini, off);
  b.maxi = __shfl_down_sync(0xffffffffu, a.maxi, off);
  b.absi = __shfl_down_sync(0xffffffffu, a.absi, off);
  return b;
}

__device__ __forceinline__ void store_rec(double *r, const Acc &a) {
#pragma unroll
  for (int j = 0; j < NSUM; ++j) r[j] = a.s[j];
  r[E_MIN_V] = a.minv;
  r[E_MIN_I] = __longlong_as_double(a.mini);
  r[E_MAX_V] = a.maxv;
  r[E_MAX_I] = __longlong_as_double(a.maxi);
  r[E_ABS_V] = a.absv;
  r[E_ABS_I] = __longlong_as_double(a.absi);
}

__device__ __forceinline__ void load_rec(Acc &a, const double *r) {
#pragma unroll
  for (int j = 0; j < NSUM; ++j) a.s[j] = r[j];
  a.minv = r[E_MIN_V];
  a.mini = __double_as_longlong(r[E_MIN_I]);
  a.maxv = r[E_MAX_V];
  a.maxi = __double_as_longlong(r[E_MAX_I]);
  a.absv = r[E_ABS_V];
  a.absi = __double_as_longlong(r[E_ABS_I]);
}

// Fixed-order block reduction over `nwarps` warps (tid: linear thread index);
// the block's record goes to partials[slot].
__device__ __forceinline__ void block_store_n(Acc &acc, double *partials, int tid, int nwarps, size_t slot) {
  __shared__ double sh[8][REC];
  const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    Acc o = shfl_down(acc, off);
    combine(acc, o);
  }
  if (lane == 0) store_rec(sh[warp], acc);
  __syncthreads();
  if (warp == 0) {
    Acc a;
    a.init();
    if (lane < nwarps) load_rec(a, sh[lane]);
#pragma unroll
    for (int off = 4; off > 0; off >>= 1) {
      Acc o = shfl_down(a, off);
      combine(a, o);
    }
    if (lane == 0) store_rec(partials + slot * REC, a);
  }
}

// The lattice kernels' form: 2-D block of THREADS, one record per block.
__device__ __forceinline__ void block_store(Acc &acc, double *partials) {
  const size_t b = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
  block_store_n(acc, partials, threadIdx.x + TX * threadIdx.y, THREADS / 32, b);
}

// Per-site observation terms, each computed with the reference's expression
// (fieldanalysis.cpp:331-355 and 433-616).  c, p: phi and pi of the site;
// fxp, fyp, fzp: forward neighbours of phi; kidx: reference index of
// component 0 of the site.
template <int NC, int THEORY>
__device__ __forceinline__ void observe(Acc &A, const Consts &k, const double *c, const double *p,
                                        const double *fxp, const double *fyp, const double *fzp,
                                        long long kidx) {
  double l = 0.0, inter = 0.0, lphi = 0.0;  // locPhiSqr, Interaction, locPhi (fieldanalysis.cpp:434-443)
#pragma unroll
  for (int a = 0; a < NC; ++a) {
    lphi = __dadd_rn(lphi, c[a]);
    A.s[S_PHI + a] += c[a];
    A.s[S_PI + a] += p[a];
    const double c2 = __dmul_rn(c[a], c[a]);
    A.s[S_PHI2] += c2;
    A.s[S_PI2] += __dmul_rn(p[a], p[a]);
    A.s[S_PHIPI] += __dmul_rn(c[a], p[a]);
    l = __dadd_rn(l, c2);
    const double dx = __dadd_rn(fxp[a], -c[a]), dy = __dadd_rn(fyp[a], -c[a]), dz = __dadd_rn(fzp[a], -c[a]);
    A.s[S_GRAD] += __dadd_rn(__dadd_rn(div_a2(k, __dmul_rn(dx, dx)), div_a2(k, __dmul_rn(dy, dy))),
                             div_a2(k, __dmul_rn(dz, dz)));
    // per-component terms (fieldanalysis.cpp:456-508)
    double term = 0.0;
    if (THEORY == 0 || THEORY == 1 || THEORY == 4) term = __dmul_rn(k.mm_half_M, c2);
    if (THEORY == 3) term = __dmul_rn(__dmul_rn(0.5, k.mmono), c2);
    if (THEORY == 1 && a == 0) term = __dadd_rn(__dmul_rn(k.h, c[a]), term);
    inter += term;
    if (!isfinite(c[a]) || !isfinite(p[a])) A.s[S_NONFINITE] += 1.0;
    A.take_max(c[a], kidx + a);
    A.take_min(c[a], kidx + a);
  }
  const double l2 = __dmul_rn(l, l);
  A.s[S_PHI4] += l2;
  A.s[S_PHI6] += __dmul_rn(l2, l);
  // per-site terms (fieldanalysis.cpp:565-617)
  if (THEORY == 0) {
    inter += __dadd_rn(__dmul_rn(k.lm, div_by_near(k, l2, k.c24, k.r_c24)), div_by(k, __dmul_rn(l2, l), k.c720, k.r_c720, k.l_c720));
  } else if (THEORY == 1) {
    inter += __dmul_rn(k.lm, div_by_near(k, l2, k.c24, k.r_c24));
  } else if (THEORY == 2 || THEORY == 3) {
    const double arg = k.expansion ? div_by(k, __dsqrt_rn(l), k.sf_sqrtm, k.r_sf_sqrtm, k.l_sf_sqrtm)
                                   : __dsqrt_rn(div_by(k, l, k.msq, k.r_msq, k.l_msq));
    inter += __dmul_rn(k.msq2, __dsub_rn(1., cos(arg)));
  } else if (THEORY == 4) {
    inter += __dadd_rn(__dmul_rn(__dmul_rn(-k.g, lphi), l) / 6.0, __dmul_rn(k.lm, div_by_near(k, l2, k.c24, k.r_c24)));
  } else {
    const double u = k.expansion ? div_by(k, div_by(k, div_by(k, l, k.msq, k.r_msq, k.l_msq), k.sf, k.r_sf, k.l_sf), k.sf, k.r_sf, k.l_sf)
                                 : div_by(k, l, k.msq, k.r_msq, k.l_msq);
    inter += __dmul_rn(k.t5c, __dsub_rn(pow(__dadd_rn(1., u), k.p_mono), 1.));
  }
  A.s[S_INTER] += inter;
  A.take_abs(sqrt(l), kidx);
}

// Per-thread FP32 accumulation for the FP32 kernels: each sum carries a
// Kahan compensation term, and the thread's totals enter the FP64 block tree
// once, at the end of its chunk.  (GB300 runs FP64 at a small fraction of its
// FP32 rate; FP64 per-site terms would cost more than the step itself.)
struct AccF {
  float s[NSUM], c[NSUM];
  float minv, maxv, absv;
  long long mini, maxi, absi;
  __device__ void init() {
#pragma unroll
    for (int j = 0; j < NSUM; ++j) s[j] = c[j] = 0.f;
    minv = 10000000.f;
    maxv = -10000000.f;
    absv = 0.f;
    mini = maxi = absi = LLONG_MAX;
  }
  __device__ __forceinline__ void add(int j, float v) {
    const float y = __fsub_rn(v, c[j]);
    const float t = __fadd_rn(s[j], y);
    c[j] = __fsub_rn(__fsub_rn(t, s[j]), y);
    s[j] = t;
  }
  __device__ void to_double(Acc &A) const {
    A.init();
#pragma unroll
    for (int j = 0; j < NSUM; ++j) A.s[j] = (double)s[j] - (double)c[j];
    if (maxi != LLONG_MAX) A.take_max((double)maxv, maxi);
    if (mini != LLONG_MAX) A.take_min((double)minv, mini);
    if (absi != LLONG_MAX) A.take_abs((double)absv, absi);
  }
};

// FP32 form of the per-site observation terms (same quantities as observe()).
template <int NC, int THEORY>
__device__ __forceinline__ void observe_f32(AccF &A, const Consts &k, const float *c, const float *p,
                                            const float *fxp, const float *fyp, const float *fzp, long long kidx) {
  float l = 0.f, inter = 0.f, lphi = 0.f;
#pragma unroll
  for (int a = 0; a < NC; ++a) {
    lphi += c[a];
    A.add(S_PHI + a, c[a]);
    A.add(S_PI + a, p[a]);
    const float c2 = c[a] * c[a];
    A.add(S_PHI2, c2);
    A.add(S_PI2, p[a] * p[a]);
    A.add(S_PHIPI, c[a] * p[a]);
    l += c2;
    const float dx = fxp[a] - c[a], dy = fyp[a] - c[a], dz = fzp[a] - c[a];
    A.add(S_GRAD, (dx * dx + dy * dy + dz * dz) * k.inv_a2_f);
    float term = 0.f;
    if (THEORY == 0 || THEORY == 1 || THEORY == 4) term = k.mmh_f * c2;
    if (THEORY == 3) term = k.mono_half_f * c2;
    if (THEORY == 1 && a == 0) term = fmaf(k.h_f, c[a], term);
    inter += term;
    if (!isfinite(c[a]) || !isfinite(p[a])) A.s[S_NONFINITE] += 1.f;
    const long long i = kidx + a;
    // ties keep the smaller index (a thread may visit indices out of order)
    if ((c[a] > A.maxv || (c[a] == A.maxv && i < A.maxi)) && c[a] > -10000000.f) { A.maxv = c[a]; A.maxi = i; }
    if ((c[a] < A.minv || (c[a] == A.minv && i < A.mini)) && c[a] < 10000000.f) { A.minv = c[a]; A.mini = i; }
  }
  const float l2 = l * l;
  A.add(S_PHI4, l2);
  A.add(S_PHI6, l2 * l);
  if (THEORY == 0 || THEORY == 1 || THEORY == 4) inter = fmaf(k.e4_f, l2, inter);
  if (THEORY == 0) inter = fmaf(k.e6_f, l2 * l, inter);
  if (THEORY == 2 || THEORY == 3) inter = fmaf(k.msq2_f, 1.f - cosf(sqrtf(l * k.inv_m_f)), inter);
  if (THEORY == 4) inter = fmaf(-k.g6_f * lphi, l, inter);
  if (THEORY == 5) inter = fmaf(k.t5c_f, powf(fmaf(l, k.inv_m_f, 1.f), k.p_f) - 1.f, inter);
  A.add(S_INTER, inter);
  const float r = sqrtf(l);
  if ((r > A.absv || (r == A.absv && kidx < A.absi)) && r > 0.f) { A.absv = r; A.absi = kidx; }
}

// Single-component form for the TMA kernel: per-site terms go into plain FP32
// partials of the current plane (16 sites per lane), and only those partials
// enter the compensated running totals -- one Kahan update per plane instead
// of one per site.  Extrema are tracked per site.
struct PlaneF {
  float v[S_NONFINITE + 1];
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int j = 0; j <= S_NONFINITE; ++j) v[j] = 0.f;
  }
};

template <int THEORY>
__device__ __forceinline__ void observe_site(PlaneF &P, AccF &A, const Consts &k, float c, float p, float xp, float yp,
                                             float zp, long long kidx) {
  const float c2 = c * c;
  P.v[S_PHI] += c;
  P.v[S_PI] += p;
  P.v[S_PHI2] += c2;
  P.v[S_PI2] += p * p;
  P.v[S_PHIPI] += c * p;
  const float dx = xp - c, dy = yp - c, dz = zp - c;
  P.v[S_GRAD] += (dx * dx + dy * dy + dz * dz) * k.inv_a2_f;
  const float l2 = c2 * c2;
  P.v[S_PHI4] += l2;
  P.v[S_PHI6] += l2 * c2;
  float inter = k.mmh_f * c2;
  if (THEORY == 1) inter = fmaf(k.h_f, c, inter);
  inter = fmaf(k.e4_f, l2, inter);
  if (THEORY == 0) inter = fmaf(k.e6_f, l2 * c2, inter);
  P.v[S_INTER] += inter;
  if (!isfinite(c) || !isfinite(p)) P.v[S_NONFINITE] += 1.f;
  if ((c > A.maxv || (c == A.maxv && kidx < A.maxi)) && c > -10000000.f) { A.maxv = c; A.maxi = kidx; }
  if ((c < A.minv || (c == A.minv && kidx < A.mini)) && c < 10000000.f) { A.minv = c; A.mini = kidx; }
  const float r = fabsf(c);  // sqrt(phi^2) for one component
  if ((r > A.absv || (r == A.absv && kidx < A.absi)) && r > 0.f) { A.absv = r; A.absi = kidx; }
}

__device__ __forceinline__ void flush_plane(AccF &A, PlaneF &P) {
#pragma unroll
  for (int j = 0; j < S_NONFINITE; ++j) A.add(j, P.v[j]);
  A.s[S_NONFINITE] += P.v[S_NONFINITE];
  P.clear();
}

constexpr int FIN_THREADS = 256;  // sh[FIN_THREADS][REC] doubles: the 48 KB of static shared memory

// Folds block records [b0, b1) in a fixed order with one block of FIN_THREADS
// threads and forms the reference's derived quantities
// (fieldanalysis.cpp:619-638): Energy, Charge, Interaction and the per-volume
// moments of a lattice of k.N^3 sites.
// The fold of records [b0, b1) by one block of FIN_THREADS threads: strided
// per thread (two records per round, combined in record order), then a fixed
// tree; the total is left in sh[0].
__device__ __forceinline__ void fold_acc(const double *__restrict__ partials, int b0, int b1,
                                         double (*sh)[REC]) {
  const int t = threadIdx.x;
  Acc a;
  a.init();
  // two records per round, loaded before either is combined (the loads of a
  // round overlap); combined in record order
  for (int b = b0 + t; b < b1; b += 2 * FIN_THREADS) {
    Acc o, o2;
    load_rec(o, partials + (size_t)b * REC);
    const bool two = b + FIN_THREADS < b1;
    if (two) load_rec(o2, partials + (size_t)(b + FIN_THREADS) * REC);
    combine(a, o);
    if (two) combine(a, o2);
  }
  store_rec(sh[t], a);
  __syncthreads();
  for (int w = FIN_THREADS / 2; w > 0; w >>= 1) {
    if (t < w) {
      Acc x, y;
      load_rec(x, sh[t]);
      load_rec(y, sh[t + w]);
      combine(x, y);
      store_rec(sh[t], x);
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void fold_records(const double *__restrict__ partials, int b0, int b1, const Consts &k,
                             phn_averages *__restrict__ out) {
  __shared__ double sh[FIN_THREADS][REC];
  fold_acc(partials, b0, b1, sh);
  if (threadIdx.x == 0) {
    Acc r;
    load_rec(r, sh[0]);
    const double vol = (double)k.N * (double)k.N * (double)k.N;
    phn_averages o;
    o.t = 0.0;
    for (int c = 0; c < PHN_MAX_NC; ++c) {
      o.phi[c] = c < k.Nc ? r.s[S_PHI + c] / vol : 0.0;
      o.pi[c] = c < k.Nc ? r.s[S_PI + c] / vol : 0.0;
    }
    const double pi2 = r.s[S_PI2], grad = r.s[S_GRAD], inter = r.s[S_INTER];
    double charge = (0.5 * pi2 - grad / 6. - inter);
    double energy = (0.5 * pi2 + 0.5 * grad + inter);
    if (k.expansion) {  // fieldanalysis.cpp:626-629, on the sums
      const double hub = (0.5 * r.s[S_PHI2] * ((k.H0 / k.sf) * (k.H0 / k.sf)) - r.s[S_PHIPI] * k.H0 / k.sf);
      energy += hub;
      charge += hub;
    }
    o.energy = energy / vol;
    o.interaction = inter / vol;
    o.charge = charge / vol;
    o.phi2 = r.s[S_PHI2] / vol;
    o.pi2 = pi2 / vol;
    o.phi4 = r.s[S_PHI4] / vol;
    o.phi6 = r.s[S_PHI6] / vol;
    o.phipi = r.s[S_PHIPI] / vol;
    o.min_phi = r.minv;
    o.max_phi = r.maxv;
    o.max_abs_phi = r.absv;
    o.min_pos = r.mini == LLONG_MAX ? -1.0 : (double)r.mini;
    o.max_pos = r.maxi == LLONG_MAX ? -1.0 : (double)r.maxi;
    o.max_abs_pos = r.absi == LLONG_MAX ? -1.0 : (double)r.absi;
    o.gradient = grad / vol;
    o.nonfinite = r.s[S_NONFINITE];
    o.scale_factor = k.sf;
    *out = o;
  }
}

}  // namespace phn
