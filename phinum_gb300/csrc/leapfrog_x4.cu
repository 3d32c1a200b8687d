// FP32 leapfrog step with four consecutive x-sites per thread (register
// path, no shared memory): updateMomenta + updateFields (dynamics.cpp:52-194)
// for one lattice, Nc = 1, N a multiple of 32.
//
// A warp covers 128 consecutive sites of a z-plane (several rows when
// N < 128), a block W warps, an item 128 W plane sites by CZ planes that the
// block marches in z with phi(z-1), phi(z), phi(z+1) in registers.  x
// neighbours inside a thread's four sites come from registers, the two
// outside ones from scalar loads that hit the cache lines of the
// neighbouring lanes' vectors; y rows and z planes move as float4, and so do
// the stores.  The per-site arithmetic is kick_drift_f32 with the same
// operands as the other FP32 kernels, so the fields are bit-identical to
// theirs.  Items are numbered (z chunk, plane chunk); a variant either walks
// them with a persistent grid or launches one block per item.  Observation
// steps run the same variant with the moment sums of ObsX4 (one block record
// per block).
//
// KAHAN: the compensated FP32 step (PHN_FP32_KAHAN) -- phi and pi carry
// per-site compensation words (read and written as float4, never read by the
// stencil) and the kick and drift use the Kahan update of step_kahan
// (leapfrog.cu) operation for operation, so both kernels give the same bits.
#include "kick.cuh"
#include "observe.cuh"
#include "phn_internal.h"

namespace phn {

struct X4Variant {
  int w, cz;
  bool persistent;
};
constexpr X4Variant kX4Variants[] = {{8, 32, true}, {8, 16, true}, {4, 32, true}, {8, 16, false},
                                     {8, 8, false},  {4, 16, false}, {8, 32, false}};
constexpr int kNumX4Variants = 7;

// Observation sums of the x4 kernel (theories 0 and 1, one component).  The
// four sites of a thread's plane row add to plain FP32 moments with FMAs --
// sum phi, pi, phi^2, pi^2, phi pi, phi^4, phi^6 and the squared forward
// differences -- which (on grids whose threads walk many items) enter
// compensated per-thread totals every OBS_FOLD planes; the FP64 record then
// takes the gradient's 1/a^2 and the interaction as the linear combination
// of the moments that theories 0 and 1 make of it (fieldanalysis.cpp:456-579:
// mmh phi^2 + lm phi^4/(24 Nc) [+ phi^6/(720 Nc^2 Kappa^2)] [+ h phi]).
// Extrema: the plane row's maximum, minimum and largest |phi| first
// (fmaxf/fminf ignore NaN, as the reference's comparisons do), kept when
// strictly beyond the thread's running value -- a thread visits its rows in
// index order, so that keeps the first site -- with the site inside the row
// found once at the end; the block tree breaks ties by the smaller index.
// Non-finite values are counted exactly, on the rare rows whose sum of 0 x
// value is not 0.
constexpr int OBS_FOLD = 4;
enum { MOM_PHI, MOM_PI, MOM_PHI2, MOM_PI2, MOM_PHIPI, MOM_PHI4, MOM_PHI6, MOM_GRAD, NMOM };

// COMP: the thread's totals are compensated (s - c, Kahan), for grids whose
// threads walk many items; with one item per block a thread adds only
// 4 x cz sites and its plain FP32 sums go straight into the block's pair tree.
template <bool COMP>
struct ObsX4 {
  float part[NMOM];
  float s[COMP ? NMOM : 1], c[COMP ? NMOM : 1];
  int nplanes;
  float nonfinite;
  float maxv, minv, absv;
  long long maxi, mini, absi;

  __device__ __forceinline__ void init() {
#pragma unroll
    for (int j = 0; j < NMOM; ++j) part[j] = 0.f;
    if constexpr (COMP) {
#pragma unroll
      for (int j = 0; j < NMOM; ++j) s[j] = c[j] = 0.f;
    }
    nplanes = 0;
    nonfinite = 0.f;
    maxv = -10000000.f;  // CalculateExtrema's starting values (fieldanalysis.cpp:324-325)
    minv = 10000000.f;
    absv = 0.f;
    maxi = mini = absi = LLONG_MAX;
  }

  __device__ __forceinline__ void site(float c, float p, float fx, float fy, float fz) {
    const float c2 = __fmul_rn(c, c), l2 = __fmul_rn(c2, c2);
    part[MOM_PHI] = __fadd_rn(part[MOM_PHI], c);
    part[MOM_PI] = __fadd_rn(part[MOM_PI], p);
    part[MOM_PHI2] = __fadd_rn(part[MOM_PHI2], c2);
    part[MOM_PI2] = __fmaf_rn(p, p, part[MOM_PI2]);
    part[MOM_PHIPI] = __fmaf_rn(c, p, part[MOM_PHIPI]);
    part[MOM_PHI4] = __fadd_rn(part[MOM_PHI4], l2);
    part[MOM_PHI6] = __fmaf_rn(l2, c2, part[MOM_PHI6]);
    const float dx = __fsub_rn(fx, c), dy = __fsub_rn(fy, c), dz = __fsub_rn(fz, c);
    part[MOM_GRAD] = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmaf_rn(dz, dz, part[MOM_GRAD])));
  }

  __device__ __forceinline__ void fold() {
    if constexpr (COMP) {
#pragma unroll
      for (int j = 0; j < NMOM; ++j) {
        const float y = __fsub_rn(part[j], c[j]);
        const float t = __fadd_rn(s[j], y);
        c[j] = __fsub_rn(__fsub_rn(t, s[j]), y);
        s[j] = t;
        part[j] = 0.f;
      }
    }
    nplanes = 0;
  }

  // One plane row of four sites: v = phi, p = pi, xr = phi right of v.w,
  // yp, zp = phi at +y, +z; kidx = reference index of v.x.
  __device__ __forceinline__ void row(float4 v, float4 p, float xr, float4 yp, float4 zp, long long kidx) {
    site(v.x, p.x, v.y, yp.x, zp.x);
    site(v.y, p.y, v.z, yp.y, zp.y);
    site(v.z, p.z, v.w, yp.z, zp.z);
    site(v.w, p.w, xr, yp.w, zp.w);
    row_rest<false>(v, p, kidx);
  }

  // The row's non-finite count, extrema and fold, after its four sites.
  // EAGER: the site inside a row is found at once (compensated fields, whose
  // compensation words the step rewrites in place); otherwise only the row is
  // kept and resolve_sites finds the site at the end.
  template <bool EAGER>
  __device__ __forceinline__ void row_rest(float4 v, float4 p, long long kidx) {
    const float z0 = fmaf(v.x, 0.f, fmaf(v.y, 0.f, fmaf(v.z, 0.f, fmaf(v.w, 0.f, 0.f))));
    const float z1 = fmaf(p.x, 0.f, fmaf(p.y, 0.f, fmaf(p.z, 0.f, fmaf(p.w, 0.f, z0))));
    if (z1 != 0.f) {  // a NaN or an infinity in this row
      const float a[8] = {v.x, v.y, v.z, v.w, p.x, p.y, p.z, p.w};
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (!isfinite(a[j])) nonfinite += 1.f;
    }
    // the row's extrema (fmaxf / fminf ignore NaN, as the reference's
    // comparisons do); a thread visits its rows in increasing index order, so
    // a strictly larger value (smaller for the minimum) keeps the first site
    // of the thread holding it.  Only the row is kept here: the site inside it
    // is found once, in block_store.
    const float hi = fmaxf(fmaxf(v.x, v.y), fmaxf(v.z, v.w));
    if (hi > maxv) {
      maxv = hi;
      maxi = EAGER ? first_of(v, hi, kidx) : kidx;
    }
    const float lo = fminf(fminf(v.x, v.y), fminf(v.z, v.w));
    if (lo < minv) {
      minv = lo;
      mini = EAGER ? first_of(v, lo, kidx) : kidx;
    }
    const float ab = fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w)));
    if (ab > absv) {  // sqrt(phi^2) of one component
      absv = ab;
      absi = EAGER ? first_of(make_float4(fabsf(v.x), fabsf(v.y), fabsf(v.z), fabsf(v.w)), ab, kidx) : kidx;
    }
    if (++nplanes == OBS_FOLD) fold();
  }

  // (h, l) += (h2, l2), both unevaluated sums: TwoSum of the high words, the
  // low words into the error, Fast2Sum.
  __device__ static __forceinline__ void pair_add(float &h, float &l, float h2, float l2) {
    const float t = __fadd_rn(h, h2);
    const float bb = __fsub_rn(t, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(t, bb)), __fsub_rn(h2, bb));
    const float lo = __fadd_rn(e, __fadd_rn(l, l2));
    h = __fadd_rn(t, lo);
    l = __fsub_rn(lo, __fsub_rn(h, t));
  }

  // Combines another thread's totals: moments as FP32 pairs, extrema by the
  // comparisons of Acc::take_* (ties keep the smaller index).
  __device__ __forceinline__ void merge(const float *h2, const float *l2, float nf2, float mx, long long ix,
                                        float mn, long long in, float ab, long long ia, float *h, float *l) {
#pragma unroll
    for (int j = 0; j < NMOM; ++j) pair_add(h[j], l[j], h2[j], l2[j]);
    nonfinite += nf2;
    if (ix != LLONG_MAX && (mx > maxv || (mx == maxv && ix < maxi && mx > -10000000.f))) {
      maxv = mx;
      maxi = ix;
    }
    if (in != LLONG_MAX && (mn < minv || (mn == minv && in < mini && mn < 10000000.f))) {
      minv = mn;
      mini = in;
    }
    if (ia != LLONG_MAX && (ab > absv || (ab == absv && ia < absi && ab > 0.f))) {
      absv = ab;
      absi = ia;
    }
  }

  __device__ __forceinline__ void shfl_merge(float *h, float *l, int off) {
    const unsigned full = 0xffffffffu;
    float h2[NMOM], l2[NMOM];
#pragma unroll
    for (int j = 0; j < NMOM; ++j) {
      h2[j] = __shfl_down_sync(full, h[j], off);
      l2[j] = __shfl_down_sync(full, l[j], off);
    }
    const float nf2 = __shfl_down_sync(full, nonfinite, off);
    const float mx = __shfl_down_sync(full, maxv, off), mn = __shfl_down_sync(full, minv, off),
                ab = __shfl_down_sync(full, absv, off);
    const long long ix = __shfl_down_sync(full, maxi, off), in = __shfl_down_sync(full, mini, off),
                    ia = __shfl_down_sync(full, absi, off);
    merge(h2, l2, nf2, mx, ix, mn, in, ab, ia, h, l);
  }

  // The block's record: the threads' compensated totals summed as FP32 pairs
  // over the warp and then over the block's W warps in a fixed tree (no FP64
  // instruction per thread: with one block per item a 512^3 lattice has
  // 16384 blocks, and per-thread FP64 trees on GB300's narrow FP64 pipe cost
  // more than the step); one thread widens the pairs to FP64 and stores the
  // record in record()'s form.
  // The first site of a kept row that holds the row's extremum (the row's
  // values v: those the step observed).
  __device__ static __forceinline__ long long first_of(float4 v, float x, long long row) {
    return row + (v.x == x ? 0 : (v.y == x ? 1 : (v.z == x ? 2 : 3)));
  }

  // Plain FP32 fields: the site of each kept row (the input phi is not
  // written during the step).
  __device__ __forceinline__ void resolve_sites(const float *phi, long long NN) {
    auto at = [&](long long row) { return *(const float4 *)(phi + (row - NN)); };
    if (maxi != LLONG_MAX) maxi = first_of(at(maxi), maxv, maxi);
    if (mini != LLONG_MAX) mini = first_of(at(mini), minv, mini);
    if (absi != LLONG_MAX) {
      const float4 v = at(absi);
      absi = first_of(make_float4(fabsf(v.x), fabsf(v.y), fabsf(v.z), fabsf(v.w)), absv, absi);
    }
  }

  template <int THEORY, int W>
  __device__ void block_store(const Consts &k, double *partials, int tid, size_t slot) {
    struct WarpTotals {
      float h[NMOM], l[NMOM];
      float nf, mx, mn, ab;
      long long ix, in, ia;
    };
    __shared__ WarpTotals sh[W];
    if (nplanes) fold();
    float h[NMOM], l[NMOM];
#pragma unroll
    for (int j = 0; j < NMOM; ++j) {
      h[j] = COMP ? s[j] : part[j];
      l[j] = COMP ? -c[j] : 0.f;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) shfl_merge(h, l, off);
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0) {
      WarpTotals &t = sh[warp];
#pragma unroll
      for (int j = 0; j < NMOM; ++j) {
        t.h[j] = h[j];
        t.l[j] = l[j];
      }
      t.nf = nonfinite;
      t.mx = maxv;
      t.mn = minv;
      t.ab = absv;
      t.ix = maxi;
      t.in = mini;
      t.ia = absi;
    }
    __syncthreads();
    if (warp == 0) {
      // lanes past the block's warps carry empty totals
      init();
#pragma unroll
      for (int j = 0; j < NMOM; ++j) h[j] = l[j] = 0.f;
      if (lane < W) {
        const WarpTotals &t = sh[lane];
#pragma unroll
        for (int j = 0; j < NMOM; ++j) {
          h[j] = t.h[j];
          l[j] = t.l[j];
        }
        nonfinite = t.nf;
        maxv = t.mx;
        minv = t.mn;
        absv = t.ab;
        maxi = t.ix;
        mini = t.in;
        absi = t.ia;
      }
#pragma unroll
      for (int off = W / 2; off > 0; off >>= 1) shfl_merge(h, l, off);
      if (lane == 0) {
        Acc A;
        A.init();
        double m[NMOM];
#pragma unroll
        for (int j = 0; j < NMOM; ++j) m[j] = (double)h[j] + (double)l[j];
        record<THEORY>(A, k, m);
        store_rec(partials + slot * REC, A);
      }
    }
  }

  // The record from the moment totals m[] (FP64) and the extrema.
  template <int THEORY>
  __device__ __forceinline__ void record(Acc &A, const Consts &k, const double *m) const {
    A.s[S_PHI] = m[MOM_PHI];
    A.s[S_PI] = m[MOM_PI];
    A.s[S_PHI2] = m[MOM_PHI2];
    A.s[S_PI2] = m[MOM_PI2];
    A.s[S_PHIPI] = m[MOM_PHIPI];
    A.s[S_PHI4] = m[MOM_PHI4];
    A.s[S_PHI6] = m[MOM_PHI6];
    A.s[S_GRAD] = m[MOM_GRAD] * k.inv_a2;
    double inter = k.mm_half_M * m[MOM_PHI2] + (k.lm / k.c24) * m[MOM_PHI4];
    if (THEORY == 0) inter += m[MOM_PHI6] / k.c720;
    if (THEORY == 1) inter += k.h * m[MOM_PHI];
    A.s[S_INTER] = inter;
    A.s[S_NONFINITE] = (double)nonfinite;
    if (maxi != LLONG_MAX) A.take_max((double)maxv, maxi);
    if (mini != LLONG_MAX) A.take_min((double)minv, mini);
    if (absi != LLONG_MAX) A.take_abs((double)absv, absi);
  }
};

// The compensated kick and drift of one site (step_kahan's arithmetic).
__device__ __forceinline__ void kahan_site(float fk, float fd, float f, float c, float ec, float p, float ep,
                                           float &tk, float &ek, float &td, float &ed) {
  const float yk = __fsub_rn(__fmul_rn(fk, f), ep);
  tk = __fadd_rn(p, yk);
  ek = __fsub_rn(__fsub_rn(tk, p), yk);
  const float yd = __fsub_rn(__fmul_rn(fd, __fsub_rn(tk, ek)), ec);
  td = __fadd_rn(c, yd);
  ed = __fsub_rn(__fsub_rn(td, c), yd);
}

// A fused observation step with one item per block keeps 4 blocks of 8
// warps per SM (64 registers): it streams the fields like the plain step and
// needs its warps for the same latency hiding.  The other kernels give no
// minimum (0): an explicit minimum of one block raised the plain step from 48
// to 64 registers.
template <int W, int MODE, int THEORY, bool KAHAN, bool COMP>
__global__ void __launch_bounds__(32 * W, (MODE == MODE_STEP_OBS && !COMP && !KAHAN) ? 32 / W : 0) step_f32_x4(const Consts k, const float *__restrict__ phi,
                                                      float *__restrict__ phi_out, float *__restrict__ pi,
                                                      float *__restrict__ cphi, float *__restrict__ cpi, StepF s,
                                                      int cz, int nitems, double *__restrict__ partials) {
  const float fk = MODE == MODE_OBS ? 0.f : (float)s.fk;
  const float fd = MODE == MODE_OBS ? 0.f : (float)s.fd;
  const int N = k.N, NN = N * N;
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const int chunks = NN / (128 * W);
  ObsX4<COMP> obs;
  if (MODE != MODE_STEP) obs.init();
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int zc = it / chunks, qc = it - zc * chunks;
    const int q = qc * (128 * W) + 4 * tid;  // this thread's first site in the plane
    const int y = q / N, x = q - y * N;
    const int qxl = (x == 0) ? q + N - 1 : q - 1;
    const int qxr = (x + 4 == N) ? q + 4 - N : q + 4;
    const int qyp = (y + 1 == N) ? q - (N - 1) * N : q + N;
    const int qym = (y == 0) ? q + (N - 1) * N : q - N;
    const int z0 = zc * cz, z1 = min(z0 + cz, N);
    float4 cm = __ldg((const float4 *)(phi + (size_t)((z0 == 0) ? N - 1 : z0 - 1) * NN + q));
    float4 c = __ldg((const float4 *)(phi + (size_t)z0 * NN + q));
    for (int z = z0; z < z1; ++z) {
      const int zn = (z + 1 == N) ? 0 : z + 1;
      const float *pl = phi + (size_t)z * NN;
      const size_t i = (size_t)z * NN + q;
      const float4 cp = __ldg((const float4 *)(phi + (size_t)zn * NN + q));
      const float4 yp = __ldg((const float4 *)(pl + qyp));
      const float4 ym = __ldg((const float4 *)(pl + qym));
      const float xm = __ldg(pl + qxl), xp = __ldg(pl + qxr);
      const float4 p = *(const float4 *)(pi + i);
      float4 ec = make_float4(0.f, 0.f, 0.f, 0.f), ep = ec;
      if (KAHAN) {
        ec = *(const float4 *)(cphi + i);
        ep = *(const float4 *)(cpi + i);
      }
      if (MODE != MODE_STEP) {
        // observables of the represented values hi - comp (neighbours: hi only)
        const long long kidx = (long long)q + (long long)(z + 1) * NN;
        if (KAHAN) {
          const float4 v = make_float4(__fsub_rn(c.x, ec.x), __fsub_rn(c.y, ec.y), __fsub_rn(c.z, ec.z),
                                       __fsub_rn(c.w, ec.w));
          const float4 pv = make_float4(__fsub_rn(p.x, ep.x), __fsub_rn(p.y, ep.y), __fsub_rn(p.z, ep.z),
                                        __fsub_rn(p.w, ep.w));
          // forward x neighbours of the hi words, as the other kernels take them
          obs.site(v.x, pv.x, c.y, yp.x, cp.x);
          obs.site(v.y, pv.y, c.z, yp.y, cp.y);
          obs.site(v.z, pv.z, c.w, yp.z, cp.z);
          obs.site(v.w, pv.w, xp, yp.w, cp.w);
          obs.template row_rest<true>(v, pv, kidx);
        } else {
          obs.row(c, p, xp, yp, cp, kidx);
        }
      }
      if (MODE != MODE_OBS) {
        if (KAHAN) {
          const float inv = k.inv_a2_f;
          float4 tk, ek, td, ed;
          kahan_site(fk, fd, force_f32<THEORY>(k, lap_diff_f32(c.x, xm, c.y, ym.x, yp.x, cm.x, cp.x, inv), c.x,
                                               __fmul_rn(c.x, c.x)),
                     c.x, ec.x, p.x, ep.x, tk.x, ek.x, td.x, ed.x);
          kahan_site(fk, fd, force_f32<THEORY>(k, lap_diff_f32(c.y, c.x, c.z, ym.y, yp.y, cm.y, cp.y, inv), c.y,
                                               __fmul_rn(c.y, c.y)),
                     c.y, ec.y, p.y, ep.y, tk.y, ek.y, td.y, ed.y);
          kahan_site(fk, fd, force_f32<THEORY>(k, lap_diff_f32(c.z, c.y, c.w, ym.z, yp.z, cm.z, cp.z, inv), c.z,
                                               __fmul_rn(c.z, c.z)),
                     c.z, ec.z, p.z, ep.z, tk.z, ek.z, td.z, ed.z);
          kahan_site(fk, fd, force_f32<THEORY>(k, lap_diff_f32(c.w, c.z, xp, ym.w, yp.w, cm.w, cp.w, inv), c.w,
                                               __fmul_rn(c.w, c.w)),
                     c.w, ec.w, p.w, ep.w, tk.w, ek.w, td.w, ed.w);
          *(float4 *)(pi + i) = tk;
          *(float4 *)(cpi + i) = ek;
          *(float4 *)(phi_out + i) = td;
          *(float4 *)(cphi + i) = ed;
        } else {
          float4 pn, fn;
          kick_drift_f32<THEORY>(k, fk, fd, c.x, xm, c.y, ym.x, yp.x, cm.x, cp.x, p.x, pn.x, fn.x);
          kick_drift_f32<THEORY>(k, fk, fd, c.y, c.x, c.z, ym.y, yp.y, cm.y, cp.y, p.y, pn.y, fn.y);
          kick_drift_f32<THEORY>(k, fk, fd, c.z, c.y, c.w, ym.z, yp.z, cm.z, cp.z, p.z, pn.z, fn.z);
          kick_drift_f32<THEORY>(k, fk, fd, c.w, c.z, xp, ym.w, yp.w, cm.w, cp.w, p.w, pn.w, fn.w);
          *(float4 *)(pi + i) = pn;
          *(float4 *)(phi_out + i) = fn;
        }
      }
      cm = c;
      c = cp;
    }
  }
  if (MODE != MODE_STEP) {  // one record per block
    if (!KAHAN) obs.resolve_sites(phi, (long long)NN);
    obs.template block_store<THEORY, W>(k, partials, tid, (size_t)blockIdx.x);
  }
}

bool x4_supported(const phn_params &p) {
  return (p.precision == PHN_FP32 || p.precision == PHN_FP32_KAHAN) && p.Nc == 1 && p.N % 32 == 0 && p.N >= 32 &&
         (p.potential == 0 || p.potential == 1);
}

int x4_num_variants() { return kNumX4Variants; }

// Observation steps run a one-item-per-block grid of the plain variant's
// width with the most planes per item: every block ends in one record (a
// block tree), so the fewer and longer the items, the less that costs (at
// 512^3: 4096 records of 32 planes against 16384 of 8), and the threads'
// totals need no compensation (128 sites each).
int x4_obs_variant(int variant) {
  int best = -1;
  for (int v = 0; v < kNumX4Variants; ++v)
    if (!kX4Variants[v].persistent && kX4Variants[v].w == kX4Variants[variant].w &&
        (best < 0 || kX4Variants[v].cz > kX4Variants[best].cz))
      best = v;
  return best >= 0 ? best : variant;
}

static int x4_items(int N, const X4Variant &v) {
  const int cz = v.cz < N ? v.cz : N;
  return ((N + cz - 1) / cz) * (N * N / (128 * v.w));
}

template <int W>
static const void *x4_fn(bool kahan) {
  return kahan ? (const void *)step_f32_x4<W, MODE_STEP, 0, true, false>
               : (const void *)step_f32_x4<W, MODE_STEP, 0, false, false>;
}

int x4_grid(const phn_params &p, int variant) {
  if (!x4_supported(p) || variant < 0 || variant >= kNumX4Variants) return 0;
  const X4Variant &v = kX4Variants[variant];
  if ((p.N * p.N) % (128 * v.w) != 0) return 0;
  const int items = x4_items(p.N, v);
  if (!v.persistent) return items;
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const bool kahan = p.precision == PHN_FP32_KAHAN;
  const void *fn = v.w == 8 ? x4_fn<8>(kahan) : x4_fn<4>(kahan);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 32 * v.w, 0) != cudaSuccess || occ < 1) occ = 1;
  const int g = sms * occ;
  return g < items ? g : items;
}

template <int W, int MODE, bool COMP>
static void x4_launch_c(const Consts &k, int theory, int grid, int cz, int nitems, const float *phi,
                        float *phi_out, float *pi, float *cphi, float *cpi, StepF s, double *partials,
                        cudaStream_t st) {
  const dim3 b(32, W);
  if (cphi) {
    if (theory == 0)
      step_f32_x4<W, MODE, 0, true, COMP><<<grid, b, 0, st>>>(k, phi, phi_out, pi, cphi, cpi, s, cz, nitems,
                                                              partials);
    else
      step_f32_x4<W, MODE, 1, true, COMP><<<grid, b, 0, st>>>(k, phi, phi_out, pi, cphi, cpi, s, cz, nitems,
                                                              partials);
  } else {
    if (theory == 0)
      step_f32_x4<W, MODE, 0, false, COMP><<<grid, b, 0, st>>>(k, phi, phi_out, pi, nullptr, nullptr, s, cz, nitems,
                                                               partials);
    else
      step_f32_x4<W, MODE, 1, false, COMP><<<grid, b, 0, st>>>(k, phi, phi_out, pi, nullptr, nullptr, s, cz, nitems,
                                                               partials);
  }
}

// Observation kernels compensate the threads' totals only where a block
// walks more than one item.
template <int W, int MODE>
static cudaError_t x4_launch_t(const Consts &k, int theory, int grid, int cz, int nitems, const float *phi,
                               float *phi_out, float *pi, float *cphi, float *cpi, StepF s, double *partials,
                               cudaStream_t st) {
  if constexpr (MODE == MODE_STEP) {
    x4_launch_c<W, MODE, false>(k, theory, grid, cz, nitems, phi, phi_out, pi, cphi, cpi, s, partials, st);
  } else {
    if (grid < nitems)
      x4_launch_c<W, MODE, true>(k, theory, grid, cz, nitems, phi, phi_out, pi, cphi, cpi, s, partials, st);
    else
      x4_launch_c<W, MODE, false>(k, theory, grid, cz, nitems, phi, phi_out, pi, cphi, cpi, s, partials, st);
  }
  return cudaGetLastError();
}

cudaError_t launch_step_f32_x4(const Consts &k, int variant, int grid, int mode, const float *phi, float *phi_out,
                               float *pi, float *cphi, float *cpi, StepF s, double *partials, cudaStream_t st) {
  const X4Variant &v = kX4Variants[variant];
  const int cz = v.cz < k.N ? v.cz : k.N;
  const int nitems = x4_items(k.N, v);
#define PHN_X4(WV, MD) \
  return x4_launch_t<WV, MD>(k, k.theory, grid, cz, nitems, phi, phi_out, pi, cphi, cpi, s, partials, st)
  if (v.w == 8) {
    if (mode == MODE_STEP) PHN_X4(8, MODE_STEP);
    if (mode == MODE_STEP_OBS) PHN_X4(8, MODE_STEP_OBS);
    PHN_X4(8, MODE_OBS);
  }
  if (mode == MODE_STEP) PHN_X4(4, MODE_STEP);
  if (mode == MODE_STEP_OBS) PHN_X4(4, MODE_STEP_OBS);
  PHN_X4(4, MODE_OBS);
#undef PHN_X4
}

}  // namespace phn
