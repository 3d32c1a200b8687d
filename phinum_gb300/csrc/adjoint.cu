// Hand-written adjoint of the leapfrog (no reference counterpart: the
// reference has no derivatives).  Differentiates
//     J = sum_x rho(x) * sigmoid((rho(x) - 2 <rho>) / w)
// of the final state, rho(x) the energy density (the summand of the
// reference's Energy, fieldanalysis.cpp:437-579), with respect to the initial
// phi field, its homogeneous part, the initial pi field and the potential's
// couplings.
//
// Forward (phn_adjoint_forward): the production step kernels through an
// internal handle (bit-identical to phn_evolve), with a checkpoint of (phi, pi)
// every `every` steps.
//
// Reverse (phn_adjoint_backward): the discrete adjoint of the implemented
// update  pi' = pi + fk F(phi),  phi' = phi + fd pi',  F = Lap(phi) - V'(phi):
//     mu      = lam_pi + fd lam_phi                  (adjoint of pi')
//     lam_phi = lam_phi + fk (Lap(mu) - V''(phi) mu)
//     lam_pi  = mu
// with (phi, pi) of the earlier time reconstructed by running the step
// backwards, phi = phi' - fd pi',  pi = pi' - fk F(phi).  Reversal is exact in
// exact arithmetic but drifts in finite precision, so each segment of `every`
// steps starts from its stored checkpoint (checkpoint-and-recompute).  One
// fused kernel per reverse step reads phi', pi', lam_phi, lam_pi and writes
// the four earlier fields: 32 bytes per site in FP32.  Coupling gradients
// accumulate per block across steps in fixed slots (deterministic).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <type_traits>
#include <vector>

#include "ccl_math.h"
#include "float_pair.cuh"
#include "kick.cuh"
#include "phn_internal.h"

namespace phn {

constexpr int ADJ_TX = 32, ADJ_TY = 8, ADJ_THREADS = ADJ_TX * ADJ_TY;
constexpr int ADJ_NG = 4;  // coupling-gradient slots: c6 (phi^6 coefficient), h, M^2 term, spare

template <typename T>
struct AdjOps;
template <>
struct AdjOps<float> {
  __device__ static float fma_(float a, float b, float c) { return fmaf(a, b, c); }
};
template <>
struct AdjOps<double> {
  __device__ static double fma_(double a, double b, double c) { return fma(a, b, c); }
};

// Per-thread compensated sum (Kahan) in T; FP64 only once per thread.
template <typename T>
struct KSum {
  T s = 0, c = 0;
  __device__ __forceinline__ void add(T v) {
    const T y = v - c;
    const T t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// The potential's pieces for one component (Nc = 1), coefficients formed
// once per thread, for the one-site-per-thread reverse step (its FP64 form is
// bound by GB300's FP64 rate):
//   V'(phi)  = (mmM + lm phi^2/6 [+ phi^4 / (120 Kappa^2)]) phi [+ h]
//   V''(phi) =  mmM + lm phi^2/2 [+ 5 phi^4 / (120 Kappa^2)]
// F = Lap(phi) - V'(phi), the Laplacian given as the sum of the six
// neighbour differences (phi_nb - phi), as in the FP32 forward kernels.
template <typename T>
struct PotCoef {
  T inv_a2, l6, c6, mmM, h;
  int theory;
  // the expanding box's couplings come scaled (at_scale_factor: mmM sf^2,
  // h sf^3) but for c6, scaled here by 1/sf^2 (sf = 1 for the static box)
  __device__ explicit PotCoef(const Consts &k)
      : inv_a2((T)1 / (T)k.a2), l6((T)k.lm / (T)k.six_nc),
        c6((T)1 / ((T)k.kappa * (T)k.kappa * (T)k.c120 * (T)k.sf * (T)k.sf)), mmM((T)k.mmM), h((T)k.h),
        theory(k.theory) {}
  __device__ __forceinline__ T force(T diff_sum, T c) const {
    const T l = c * c;
    T coef = mmM + l * l6;
    if (theory == 0) coef += (l * l) * c6;
    T f = diff_sum * inv_a2 - coef * c;
    if (theory == 1) f -= h;
    return f;
  }
  __device__ __forceinline__ T vpp(T c) const {
    const T l = c * c;
    T v = mmM + (T)3 * l * l6;
    if (theory == 0) v += (T)5 * (l * l) * c6;
    return v;
  }
};

// A plain running sum (FP64 partials need no compensation over one column).
template <typename T>
struct PSum {
  T s = 0;
  __device__ __forceinline__ void add(T v) { s += v; }
  __device__ __forceinline__ double value() const { return (double)s; }
};

// Block-level sum of the two per-thread gradient partials into this
// block's slot (fixed order: warp shuffles, then the warps in order).
__device__ __forceinline__ void grad_slot_add(double g0, double g1, double *gs, int tid, int nwarps) {
  __shared__ double sh[2][32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    g0 += __shfl_down_sync(0xffffffffu, g0, off);
    g1 += __shfl_down_sync(0xffffffffu, g1, off);
  }
  if ((tid & 31) == 0) {
    sh[0][tid >> 5] = g0;
    sh[1][tid >> 5] = g1;
  }
  __syncthreads();
  if (tid == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int w = 0; w < nwarps; ++w) {
      s0 += sh[0][w];
      s1 += sh[1][w];
    }
    const size_t b = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
    gs[b * ADJ_NG + 0] += s0;
    gs[b * ADJ_NG + 1] += s1;
  }
}

// grad_slot_add for two per-thread compensated FP32 sums (value s - c): the
// warp shuffles and the sum over the warps add float pairs, and FP64 is used
// by the one thread that adds to the block's slots.  The FP64 form cost the
// FP32 reverse step a tenth of its time at 128^3: every block of the single
// wave reaches its reduction at the same moment, on GB300's narrow FP64 pipe.
__device__ __forceinline__ void grad_slot_add_f32(const KSum<float> &a, const KSum<float> &b, double *gs, int tid,
                                                  int nwarps) {
  __shared__ float sh[4][32];
  float h0 = a.s, l0 = -a.c, h1 = b.s, l1 = -b.c;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float h0n = __shfl_down_sync(0xffffffffu, h0, off), l0n = __shfl_down_sync(0xffffffffu, l0, off);
    const float h1n = __shfl_down_sync(0xffffffffu, h1, off), l1n = __shfl_down_sync(0xffffffffu, l1, off);
    fpair_add(h0, l0, h0n, l0n);
    fpair_add(h1, l1, h1n, l1n);
  }
  if ((tid & 31) == 0) {
    sh[0][tid >> 5] = h0;
    sh[1][tid >> 5] = l0;
    sh[2][tid >> 5] = h1;
    sh[3][tid >> 5] = l1;
  }
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < nwarps; ++w) {
      fpair_add(h0, l0, sh[0][w], sh[1][w]);
      fpair_add(h1, l1, sh[2][w], sh[3][w]);
    }
    const size_t blk = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
    gs[blk * ADJ_NG + 0] += (double)h0 + (double)l0;
    gs[blk * ADJ_NG + 1] += (double)h1 + (double)l1;
  }
}

// One reverse step, one site per thread (any N; the FP64 path).
// phi1, pi1: state after the step; lphi, lpi: adjoints at that time.  Writes
// phi0, pi0 (state before) and lphi0, lpi0 (adjoints before).  Gradient slots:
// gs[block][j] += this step's coupling terms.
template <typename T>
__global__ void __launch_bounds__(ADJ_THREADS) adjoint_step(const T *__restrict__ phi1, const T *__restrict__ pi1,
                                                            const T *__restrict__ lphi, const T *__restrict__ lpi,
                                                            T *__restrict__ phi0, T *__restrict__ pi0,
                                                            T *__restrict__ lphi0, T *__restrict__ lpi0,
                                                            const Consts k, const T fk, const T fd, const double gk6,
                                                            const double gkh, const int cz, double *__restrict__ gs) {
  const int N = k.N;
  const int x = blockIdx.x * ADJ_TX + threadIdx.x, y = blockIdx.y * ADJ_TY + threadIdx.y;
  const int z0 = blockIdx.z * cz, z1 = min(z0 + cz, N);
  const size_t NN = (size_t)N * N;
  // sum_z mu phi^5 and sum_z mu; the step's factors -6 fk and -fk apply once
  using Sum = typename std::conditional<std::is_same<T, double>::value, PSum<T>, KSum<T>>::type;
  Sum k_c6, k_h;
  const PotCoef<T> pc_k(k);
  static_assert(ADJ_TX == 32, "a warp spans one row segment of 32 sites");
  const bool warp_rows = (N & 31) == 0;
  if (x < N && y < N && z0 < z1) {
    const int xp = (x + 1 == N) ? 0 : x + 1, xm = (x == 0) ? N - 1 : x - 1;
    const int yp = (y + 1 == N) ? 0 : y + 1, ym = (y == 0) ? N - 1 : y - 1;
    const size_t col = (size_t)y * N + x;
    auto rphi = [&](size_t i) { return AdjOps<T>::fma_(-fd, pi1[i], phi1[i]); };
    auto rmu = [&](size_t i) { return AdjOps<T>::fma_(fd, lphi[i], lpi[i]); };
    const int zm0 = (z0 == 0) ? N - 1 : z0 - 1;
    T pm = rphi((size_t)zm0 * NN + col), pc = rphi((size_t)z0 * NN + col);
    T mm = rmu((size_t)zm0 * NN + col), mc = rmu((size_t)z0 * NN + col);
    const T inv_a2 = pc_k.inv_a2;
    for (int z = z0; z < z1; ++z) {
      const int zn = (z + 1 == N) ? 0 : z + 1;
      const size_t pl = (size_t)z * NN, i = pl + col;
      const T pn = rphi((size_t)zn * NN + col), mn = rmu((size_t)zn * NN + col);
      const size_t ixp = pl + (size_t)y * N + xp, ixm = pl + (size_t)y * N + xm;
      const size_t iyp = pl + (size_t)yp * N + x, iym = pl + (size_t)ym * N + x;
      // x neighbours: from the next / previous lane where a warp spans 32
      // sites of one row (N a multiple of 32: whole warps active), else
      // reconstructed here -- the same values either way
      T pxp, pxm, mxp, mxm;
      if (warp_rows) {
        const int lane = threadIdx.x;
        pxp = __shfl_down_sync(0xffffffffu, pc, 1);
        pxm = __shfl_up_sync(0xffffffffu, pc, 1);
        mxp = __shfl_down_sync(0xffffffffu, mc, 1);
        mxm = __shfl_up_sync(0xffffffffu, mc, 1);
        if (lane == 31) {
          pxp = rphi(ixp);
          mxp = rmu(ixp);
        }
        if (lane == 0) {
          pxm = rphi(ixm);
          mxm = rmu(ixm);
        }
      } else {
        pxp = rphi(ixp);
        pxm = rphi(ixm);
        mxp = rmu(ixp);
        mxm = rmu(ixm);
      }
      const T dphi = (((pxp - pc) + (pxm - pc)) + ((rphi(iyp) - pc) + (rphi(iym) - pc))) + ((pn - pc) + (pm - pc));
      const T pi_before = AdjOps<T>::fma_(-fk, pc_k.force(dphi, pc), pi1[i]);
      const T dmu = (((mxp - mc) + (mxm - mc)) + ((rmu(iyp) - mc) + (rmu(iym) - mc))) + ((mn - mc) + (mm - mc));
      const T lphi_before = AdjOps<T>::fma_(fk, dmu * inv_a2 - pc_k.vpp(pc) * mc, lphi[i]);
      phi0[i] = pc;
      pi0[i] = pi_before;
      lphi0[i] = lphi_before;
      lpi0[i] = mc;
      // dF/dc6 = -6 phi^5 ; dF/dh = -1   (kick pi' = pi + fk F)
      const T p2 = pc * pc;
      k_c6.add(mc * (p2 * p2 * pc));
      k_h.add(mc);
      pm = pc;
      pc = pn;
      mm = mc;
      mc = mn;
    }
  }
  grad_slot_add(-6.0 * gk6 * k_c6.value(), -gkh * k_h.value(), gs, threadIdx.x + ADJ_TX * threadIdx.y,
                ADJ_THREADS / 32);
}

// The same reverse step for FP32, four consecutive x-sites per thread
// (N a multiple of 4): 16-byte loads and stores, x neighbours inside the
// thread plus one scalar per side, y rows and z planes as float4.  The
// reconstruction pi = pi' - fk F(phi) uses the forward kick's own FP32 force
// (kick.cuh) and coefficients; the theory is a template parameter, and
// theory 0 is held to 80 registers (three blocks of 8 warps per SM).
__device__ __forceinline__ float4 f4fma(float a, float4 b, float4 c) {
  return make_float4(fmaf(a, b.x, c.x), fmaf(a, b.y, c.y), fmaf(a, b.z, c.z), fmaf(a, b.w, c.w));
}
__device__ __forceinline__ float f4get(const float4 &v, int e) {
  return e == 0 ? v.x : (e == 1 ? v.y : (e == 2 ? v.z : v.w));
}
__device__ __forceinline__ void f4set(float4 &v, int e, float x) {
  if (e == 0) v.x = x;
  else if (e == 1) v.y = x;
  else if (e == 2) v.z = x;
  else v.w = x;
}

template <int THEORY>
__global__ void __launch_bounds__(ADJ_THREADS, THEORY == 0 ? 3 : 0) adjoint_step_x4(const float *__restrict__ phi1,
                                                               const float *__restrict__ pi1,
                                                               const float *__restrict__ lphi,
                                                               const float *__restrict__ lpi, float *__restrict__ phi0,
                                                               float *__restrict__ pi0, float *__restrict__ lphi0,
                                                               float *__restrict__ lpi0, const Consts k, const float fk,
                                                               const float fd, const float gk6, const float gkh,
                                                               const int cz, double *__restrict__ gs) {
  const int N = k.N;
  const int x0 = (blockIdx.x * ADJ_TX + threadIdx.x) * 4, y = blockIdx.y * ADJ_TY + threadIdx.y;
  const int z0 = blockIdx.z * cz, z1 = min(z0 + cz, N);
  const size_t NN = (size_t)N * N;
  KSum<float> k_c6, k_h;
  if (x0 < N && y < N && z0 < z1) {
    const int xl = (x0 == 0) ? N - 1 : x0 - 1, xr = (x0 + 4 == N) ? 0 : x0 + 4;
    const int yp = (y + 1 == N) ? 0 : y + 1, ym = (y == 0) ? N - 1 : y - 1;
    const size_t col = (size_t)y * N + x0;
    auto ld4 = [&](const float *f, size_t i) { return *(const float4 *)(f + i); };
    auto rphi4 = [&](size_t i) { return f4fma(-fd, ld4(pi1, i), ld4(phi1, i)); };
    auto rmu4 = [&](size_t i) { return f4fma(fd, ld4(lphi, i), ld4(lpi, i)); };
    auto rphi1 = [&](size_t i) { return fmaf(-fd, pi1[i], phi1[i]); };
    auto rmu1 = [&](size_t i) { return fmaf(fd, lphi[i], lpi[i]); };
    const int zm0 = (z0 == 0) ? N - 1 : z0 - 1;
    float4 pm = rphi4((size_t)zm0 * NN + col), mm = rmu4((size_t)zm0 * NN + col);
    size_t ic = (size_t)z0 * NN + col;
    float4 pc = rphi4(ic), mc = rmu4(ic), pic = ld4(pi1, ic), lphic = ld4(lphi, ic);
    // V''(phi) = mmM + 3 c4 phi^2 [+ 5 c6 phi^4] with the forward kick's FP32
    // coefficients (parameter-space constants: no per-site FP64 conversion)
    const float c4x3 = 3.f * k.c4_f, c6x5 = 5.f * k.c6_f;
    for (int z = z0; z < z1; ++z) {
      const int zn = (z + 1 == N) ? 0 : z + 1;
      const size_t pl = (size_t)z * NN, i = pl + col, in = (size_t)zn * NN + col;
      const float4 pn = rphi4(in), mn = rmu4(in), pin = ld4(pi1, in), lphin = ld4(lphi, in);
      const size_t iyp = pl + (size_t)yp * N + x0, iym = pl + (size_t)ym * N + x0;
      const float4 pyp = rphi4(iyp), pym = rphi4(iym), myp = rmu4(iyp), mym = rmu4(iym);
      const size_t ixl = pl + (size_t)y * N + xl, ixr = pl + (size_t)y * N + xr;
      const float pxl = rphi1(ixl), pxr = rphi1(ixr), mxl = rmu1(ixl), mxr = rmu1(ixr);
      float4 o_phi, o_pi, o_lphi;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float c = f4get(pc, e), m = f4get(mc, e);
        const float cxm = e == 0 ? pxl : f4get(pc, e - 1), cxp = e == 3 ? pxr : f4get(pc, e + 1);
        const float mxm = e == 0 ? mxl : f4get(mc, e - 1), mxp = e == 3 ? mxr : f4get(mc, e + 1);
        const float lap = lap_diff_f32(c, cxm, cxp, f4get(pym, e), f4get(pyp, e), f4get(pm, e), f4get(pn, e),
                                       k.inv_a2_f);
        const float lmu = lap_diff_f32(m, mxm, mxp, f4get(mym, e), f4get(myp, e), f4get(mm, e), f4get(mn, e),
                                       k.inv_a2_f);
        const float c2 = __fmul_rn(c, c);
        const float vpp = THEORY == 0 ? fmaf(c2, fmaf(c2, c6x5, c4x3), k.mmM_f) : fmaf(c2, c4x3, k.mmM_f);
        f4set(o_phi, e, c);
        f4set(o_pi, e, fmaf(-fk, force_f32<THEORY>(k, lap, c, c2), f4get(pic, e)));
        f4set(o_lphi, e, fmaf(fk, fmaf(-vpp, m, lmu), f4get(lphic, e)));
        k_c6.add(gk6 * m * (-6.f * (c2 * c2 * c)));
        k_h.add(-gkh * m);
      }
      *(float4 *)(phi0 + i) = o_phi;
      *(float4 *)(pi0 + i) = o_pi;
      *(float4 *)(lphi0 + i) = o_lphi;
      *(float4 *)(lpi0 + i) = mc;
      pm = pc;
      pc = pn;
      mm = mc;
      mc = mn;
      pic = pin;
      lphic = lphin;
    }
  }
  grad_slot_add_f32(k_c6, k_h, gs, threadIdx.x + ADJ_TX * threadIdx.y, ADJ_THREADS / 32);
}

// Grid of the reverse kernel (x4: a block covers 128 x-sites).  Cost model:
// whole waves of the resident capacity times the planes a block handles
// plus its fixed overhead (two z-halo planes, the gradient reduction); every
// plane count from 1 to 64 is a candidate, so that the grid can fill one wave
// of resident blocks.  At 128^3 (three blocks of 8 warps per SM) that is 5
// planes, 416 blocks: 13.3 ms per 1000 reverse steps, against 14.8 ms for 8
// planes (256 blocks, 0.56 of a wave), 14.7 ms for 6 and 17.1 ms for 4 (512
// blocks, a second wave).  A 64-register cap for four blocks per SM measured
// slower (spills).  PHN_ADJ_CZ overrides the planes per block (tuning).
static Grid adjoint_grid(int N, bool x4) {
  Grid g;
  g.block = dim3(ADJ_TX, ADJ_TY, 1);
  const int xs = x4 ? 4 * ADJ_TX : ADJ_TX;
  const int gx = (N + xs - 1) / xs, gy = (N + ADJ_TY - 1) / ADJ_TY;
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (x4)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, adjoint_step_x4<0>, ADJ_THREADS, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, adjoint_step<double>, ADJ_THREADS, 0);
  const long long resident = (long long)sms * (occ > 0 ? occ : 1);
  int best_cz = 8;
  double best_cost = 1e300;
  for (int cz = 1; cz <= 64 && cz <= N; ++cz) {
    const long long blocks = (long long)gx * gy * ((N + cz - 1) / cz);
    const double cost = (double)((blocks + resident - 1) / resident) * (cz + 2.0);
    if (cost < best_cost) {
      best_cost = cost;
      best_cz = cz;
    }
  }
  const char *env = getenv("PHN_ADJ_CZ");
  if (env && atoi(env) > 0) best_cz = atoi(env);
  g.cz = best_cz;
  g.grid = dim3(gx, gy, (N + best_cz - 1) / best_cz);
  g.nblocks = gx * gy * g.grid.z;
  return g;
}

// ---------------------------------------------------------------- objective
// J = sum_x rho(x) s(x), s = sigmoid((rho(x) - 2 <rho>) / w), and its seed
// g = dJ/drho, in three passes with FP64 per-site terms.  Each pass leaves one
// sum per block in part[]; the next pass folds those on the device in a fixed
// order (the same in every block), so nothing returns to the host until J is
// read back and the result is identical run to run.
constexpr int OBJ_THREADS = 256;

__device__ __forceinline__ double sigmoid(double u) { return 1.0 / (1.0 + exp(-u)); }

// Fixed-order block sum of one value per thread; the result is valid in
// thread 0.  Every thread of the block calls it.
__device__ double obj_block_sum(double v) {
  __shared__ double sh[OBJ_THREADS / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < OBJ_THREADS / 32; ++w) s += sh[w];
  __syncthreads();
  return s;
}

// Sum of part[0..n): lane l adds part[l], part[l+32], ... in sequence, then a
// butterfly; the same bits in every block.  Every thread of the block calls it.
__device__ double obj_fold(const double *part, int n) {
  __shared__ double r;
  if (threadIdx.x < 32) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) s += part[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (threadIdx.x == 0) r = s;
  }
  __syncthreads();
  const double v = r;
  __syncthreads();
  return v;
}

// Pass 1: rho(x) from T fields (the summand of the reference's Energy:
// pi^2/2 + forward-difference gradient energy + V) and block sums of rho.
// x, y, z of site i (i < 2^31) by multiply-high division (ccl_math.h), not
// 64-bit divisions.
__device__ __forceinline__ void obj_xyz(const DivN &q, int N, size_t i, int &x, int &y, int &z) {
  const unsigned row = div_n(q, (unsigned)i), zz = div_n(q, row);
  x = (int)((unsigned)i - row * (unsigned)N);
  y = (int)(row - zz * (unsigned)N);
  z = (int)zz;
}

template <typename T>
__global__ void __launch_bounds__(OBJ_THREADS) obj_rho(const T *__restrict__ phi, const T *__restrict__ pi,
                                                       const Consts k, const DivN dn, double *__restrict__ rho,
                                                       double *__restrict__ part) {
  const int N = k.N;
  const size_t NN = (size_t)N * N, V = NN * N;
  const double ia2 = 1.0 / k.a2, i24 = 1.0 / k.c24, i720 = 1.0 / k.c720;
  double acc = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < V; i += (size_t)gridDim.x * blockDim.x) {
    int x, y, z;
    obj_xyz(dn, N, i, x, y, z);
    const double c = phi[i], p = pi[i];
    const double fx = phi[i - x + (x + 1 == N ? 0 : x + 1)];
    const double fy = phi[(size_t)z * NN + (size_t)(y + 1 == N ? 0 : y + 1) * N + x];
    const double fz = phi[(size_t)(z + 1 == N ? 0 : z + 1) * NN + (size_t)y * N + x];
    const double c2 = c * c, c4 = c2 * c2;
    const double grad = ((fx - c) * (fx - c) + (fy - c) * (fy - c) + (fz - c) * (fz - c)) * ia2;
    double v = k.mm_half_M * c2 + k.lm * (c4 * i24);
    if (k.theory == 0) v += c4 * c2 * i720;
    if (k.theory == 1) v += k.h * c;
    double kin = 0.5 * p * p;
    if (k.expansion) {  // fieldanalysis.cpp:626-629: + (H0/sf)^2 phi^2 / 2 - phi pi H0/sf
      const double hub = k.H0 / k.sf;
      kin += 0.5 * (hub * hub) * c2 - c * p * hub;
    }
    const double r = kin + 0.5 * grad + v;
    rho[i] = r;
    acc += r;
  }
  const double s = obj_block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Pass 2: <rho> from pass 1; s(x) into sg; block sums of rho s (J) and of
// rho s (1 - s) (S, the seed's coupling through the mean).
__global__ void __launch_bounds__(OBJ_THREADS) obj_sigmoid(const double *__restrict__ rho, size_t V, double w,
                                                           double *__restrict__ sg, double *__restrict__ part,
                                                           int nb) {
  const double mean = obj_fold(part, nb) / (double)V;
  const double iw = 1.0 / w;
  double aj = 0.0, as = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < V; i += (size_t)gridDim.x * blockDim.x) {
    const double r = rho[i], s = sigmoid((r - 2.0 * mean) * iw);
    sg[i] = s;
    aj += r * s;
    as += r * s * (1.0 - s);
  }
  const double sj = obj_block_sum(aj), ss = obj_block_sum(as);
  if (threadIdx.x == 0) {
    part[nb + blockIdx.x] = sj;
    part[2 * nb + blockIdx.x] = ss;
  }
}

// Pass 3: g(x) = dJ/drho(x) = s + rho s (1 - s) / w - 2 S / (w V), written
// over s; block 0 stores <rho>, J, S in res[0..2].
__global__ void __launch_bounds__(OBJ_THREADS) obj_seed(const double *__restrict__ rho, size_t V, double w,
                                                        double *__restrict__ g, const double *__restrict__ part,
                                                        int nb, double *__restrict__ res) {
  const double S = obj_fold(part + 2 * nb, nb);
  const double iw = 1.0 / w, corr = -2.0 * S * iw / (double)V;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < V; i += (size_t)gridDim.x * blockDim.x) {
    const double r = rho[i], s = g[i];
    g[i] = s + r * s * (1.0 - s) * iw + corr;
  }
  if (blockIdx.x == 0) {
    const double sr = obj_fold(part, nb), sj = obj_fold(part + nb, nb);
    if (threadIdx.x == 0) {
      res[0] = sr / (double)V;
      res[1] = sj;
      res[2] = S;
    }
  }
}

// Adjoint of J at the final state (lam = dJ/d(phi, pi)):
//   lam_pi = g pi
//   lam_phi = g (-sum_d (phi(x+d) - phi(x)) / a^2 + V'(phi)) + sum_d g(x-d) (phi(x) - phi(x-d)) / a^2
// and, in the same pass, block sums of the direct coupling terms
// dJ/dc6 = sum g phi^6 and dJ/dh = sum g phi into part[0..nb), part[nb..2nb).
template <typename T, typename L>
__global__ void __launch_bounds__(OBJ_THREADS) obj_adjoint_init(const T *__restrict__ phi, const T *__restrict__ pi,
                                                                const double *__restrict__ g, const Consts k,
                                                                const DivN dn, L *__restrict__ lphi,
                                                                L *__restrict__ lpi, double *__restrict__ part,
                                                                int nb) {
  const int N = k.N;
  const size_t NN = (size_t)N * N, V = NN * N;
  const double ia2 = 1.0 / k.a2, i720 = 1.0 / k.c720, l6 = k.lm * (24.0 / k.c24) / 6.0;
  double a6 = 0.0, ah = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < V; i += (size_t)gridDim.x * blockDim.x) {
    int x, y, z;
    obj_xyz(dn, N, i, x, y, z);
    const size_t ixp = i - x + (x + 1 == N ? 0 : x + 1), ixm = i - x + (x == 0 ? N - 1 : x - 1);
    const size_t iyp = (size_t)z * NN + (size_t)(y + 1 == N ? 0 : y + 1) * N + x;
    const size_t iym = (size_t)z * NN + (size_t)(y == 0 ? N - 1 : y - 1) * N + x;
    const size_t izp = (size_t)(z + 1 == N ? 0 : z + 1) * NN + (size_t)y * N + x;
    const size_t izm = (size_t)(z == 0 ? N - 1 : z - 1) * NN + (size_t)y * N + x;
    const double c = phi[i], gi = g[i];
    const double fwd = ((double)phi[ixp] - c) + ((double)phi[iyp] - c) + ((double)phi[izp] - c);
    const double bwd = g[ixm] * (c - (double)phi[ixm]) + g[iym] * (c - (double)phi[iym]) +
                       g[izm] * (c - (double)phi[izm]);
    const double c2 = c * c;
    double vp = 2.0 * k.mm_half_M * c + l6 * c2 * c;
    if (k.theory == 0) vp += 6.0 * c2 * c2 * c * i720;
    if (k.theory == 1) vp += k.h;
    double dk_phi = 0.0, dk_pi = (double)pi[i];  // the kinetic term's derivatives
    if (k.expansion) {
      const double hub = k.H0 / k.sf;
      dk_phi = (hub * hub) * c - (double)pi[i] * hub;
      dk_pi -= c * hub;
    }
    lphi[i] = (L)(gi * (-fwd * ia2 + vp + dk_phi) + bwd * ia2);
    lpi[i] = (L)(gi * dk_pi);
    a6 += gi * (c2 * c2 * c2);
    ah += gi * c;
  }
  const double s6 = obj_block_sum(a6), sh = obj_block_sum(ah);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s6;
    part[nb + blockIdx.x] = sh;
  }
}

// FP64 forward state -> FP32 checkpoint (round to nearest)
__global__ void narrow_f64(const double *__restrict__ src, float *__restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

__global__ void gs_zero(double *gs, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) gs[i] = 0.0;
}

}  // namespace phn

using namespace phn;

struct phn_adjoint {
  phn_params p;
  Consts k;
  int nsteps, every, nseg;
  double w;
  size_t V, elem;          // elem: bytes of a checkpoint / reverse-sweep value
  size_t fwd_elem;         // bytes of a forward value (8 for an FP64 forward)
  phn_handle *fwd;
  void *ckpt;              // (nseg + 1) x {phi, pi}
  void *rphi[2], *rpi[2], *lphi[2], *lpi[2];
  double *rho, *g;         // per-site FP64 scratch: rho, then s / the seed g
  double *sums;            // block sums [3][sum_blocks] + 4 results (<rho>, J, S)
  double *h_res;           // pinned host copy of the results
  double *gs;              // gradient slots [blocks][ADJ_NG]
  int sum_blocks;
  std::vector<double> fk, fd;  // clock factors of each forward step
  std::vector<double> sfk;     // the scale factor of each step's kick (1 for the static box)
  double sf_fin;               // the scale factor of the final state (J's)
  bool forward_done;
  double J, mean, S;
  cudaEvent_t ev0, ev1;
  double fwd_ms, bwd_ms;
  cudaGraphExec_t sweep;  // the captured reverse sweep
  bool graph_ok;
  int final_cur;          // buffer parity of the adjoint after the sweep
  // forward in FP32 pairs (phn_adjoint_set_forward_precision(PHN_FP32_PAIR)):
  // phi (hi, lo) double-buffered, pi (hi, lo), the final state widened to
  // FP64 for the objective, and an FP64 reference-layout staging buffer
  bool pair;
  float *pph[2], *ppl[2], *pqh, *pql;
  double *pfin, *pstage;
  cudaGraphExec_t pgraph;  // the pair forward's steps and checkpoints, captured once
  bool pgraph_ok;
};

static void adj_free(phn_adjoint *a) {
  if (!a) return;
  if (a->fwd) phn_destroy(a->fwd);
  cudaFree(a->ckpt);
  for (int i = 0; i < 2; ++i) {
    cudaFree(a->rphi[i]);
    cudaFree(a->rpi[i]);
    cudaFree(a->lphi[i]);
    cudaFree(a->lpi[i]);
  }
  cudaFree(a->rho);
  cudaFree(a->g);
  cudaFree(a->sums);
  if (a->h_res) cudaFreeHost(a->h_res);
  cudaFree(a->gs);
  for (int i = 0; i < 2; ++i) {
    cudaFree(a->pph[i]);
    cudaFree(a->ppl[i]);
  }
  cudaFree(a->pqh);
  cudaFree(a->pql);
  cudaFree(a->pfin);
  cudaFree(a->pstage);
  if (a->pgraph_ok) cudaGraphExecDestroy(a->pgraph);
  if (a->ev0) cudaEventDestroy(a->ev0);
  if (a->ev1) cudaEventDestroy(a->ev1);
  if (a->graph_ok) cudaGraphExecDestroy(a->sweep);
  delete a;
}

#define CKA(call)                                        \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_error(e_, #call); \
  } while (0)

// J and its seed g on the current forward state (phi, pi device pointers);
// <rho>, J, S are copied to the pinned h_res (read after the stream syncs).
// The clock of one evolve() as the handle runs it (dynamics.cpp:196-237):
// the kick factor, the drift factor and the kick's scale factor (conformal
// times and sqrt(1 + 2 H0 tau) in the expanding box, 1 in the static one).
struct AdjClock {
  double tau, dtau, lm, lf, lmc, lfc, tc, H0;
  bool ex;
  void step(double &fk, double &fd, double &sfk) {
    tau += 0.5 * dtau;
    if (ex) {
      tc = (sqrt(1. + 2. * H0 * tau) - 1.) / H0;
      sfk = sqrt(1. + 2. * H0 * tau);
      fk = tc - lmc;
    } else {
      sfk = 1.0;
      fk = tau - lm;
    }
    lm = tau;
    lmc = ex ? tc : tau;
    tau += 0.5 * dtau;
    if (ex) {
      tc = (sqrt(1. + 2. * H0 * tau) - 1.) / H0;
      fd = tc - lfc;
    } else {
      fd = tau - lf;
      tc = tau;
    }
    lf = tau;
    lfc = tc;
  }
  double sf() const { return ex ? sqrt(1. + 2. * H0 * tau) : 1.0; }
};

// The couplings of the final state (J) and of step n's kick.
static Consts final_consts(const phn_adjoint *a) {
  return a->p.expanding ? at_scale_factor(a->k, a->sf_fin) : a->k;
}
static Consts step_consts(const phn_adjoint *a, int n) {
  return a->p.expanding ? at_scale_factor(a->k, a->sfk[n]) : a->k;
}

template <typename T>
static int objective(phn_adjoint *a, const T *phi, const T *pi, cudaStream_t st) {
  const int nb = a->sum_blocks;
  double *res = a->sums + 3 * nb;
  obj_rho<T><<<nb, OBJ_THREADS, 0, st>>>(phi, pi, final_consts(a), make_divn((unsigned)a->k.N), a->rho, a->sums);
  obj_sigmoid<<<nb, OBJ_THREADS, 0, st>>>(a->rho, a->V, a->w, a->g, a->sums, nb);
  obj_seed<<<nb, OBJ_THREADS, 0, st>>>(a->rho, a->V, a->w, a->g, a->sums, nb, res);
  CKA(cudaGetLastError());
  CKA(cudaMemcpyAsync(a->h_res, res, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  return PHN_OK;
}

extern "C" {

int phn_adjoint_create(const phn_params *params, int nsteps, int every, double width, phn_adjoint **out) {
  if (!out || nsteps < 1 || every < 1 || nsteps % every != 0 || !(width > 0.0))
    return set_error(PHN_ERR_INVALID, "nsteps must be a positive multiple of every; width > 0");
  *out = nullptr;
  int r = validate_params(params);
  if (r) return r;
  if (params->Nc != 1 || params->precision == PHN_FP32_KAHAN || params->potential > 1)
    return set_error(PHN_ERR_UNSUPPORTED, "adjoint: theories 0 and 1, Nc = 1, FP32 or FP64");
  phn_adjoint *a = new phn_adjoint();
  a->p = *params;
  a->k = make_consts(params);
  a->nsteps = nsteps;
  a->every = every;
  a->nseg = nsteps / every;
  a->w = width;
  a->V = (size_t)params->N * params->N * params->N;
  a->elem = params->precision == PHN_FP64 ? 8 : 4;
  a->fwd_elem = a->elem;
  r = phn_create(params, &a->fwd);
  if (r) {
    adj_free(a);
    return r;
  }
  const size_t fb = a->V * a->elem;
  cudaError_t e = cudaMalloc(&a->ckpt, (size_t)(a->nseg + 1) * 2 * fb);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
    e = cudaMalloc(&a->rphi[i], fb);
    if (e == cudaSuccess) e = cudaMalloc(&a->rpi[i], fb);
    if (e == cudaSuccess) e = cudaMalloc(&a->lphi[i], fb);
    if (e == cudaSuccess) e = cudaMalloc(&a->lpi[i], fb);
  }
  a->sum_blocks = 152 * 4;
  if (e == cudaSuccess) e = cudaMalloc(&a->rho, a->V * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&a->g, a->V * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&a->sums, (3 * (size_t)a->sum_blocks + 4) * sizeof(double));
  if (e == cudaSuccess) e = cudaHostAlloc((void **)&a->h_res, 4 * sizeof(double), cudaHostAllocDefault);
  const Grid gr = adjoint_grid(params->N, params->precision != PHN_FP64 && params->N % 4 == 0);
  if (e == cudaSuccess) e = cudaMalloc(&a->gs, (size_t)gr.nblocks * ADJ_NG * sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreate(&a->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&a->ev1);
  if (e != cudaSuccess) {
    r = cuda_error(e, "adjoint buffers");
    adj_free(a);
    return r;
  }
  *out = a;
  return PHN_OK;
}

int phn_adjoint_destroy(phn_adjoint *a) {
  adj_free(a);
  return PHN_OK;
}

// The forward solve in FP32 pairs: the clock of dynamics.cpp:28-50,196-213
// on the host (the factors the handle would use), one pair step per evolve(),
// FP32 checkpoints from the high words (the pair's rounding to FP32), and J
// with its seed on the final state widened to FP64.
static int forward_pair(phn_adjoint *a, const double *Phi0, const double *Pi0) {
  phn_handle *h = a->fwd;
  cudaStream_t st = h->stream;
  const int N = a->p.N;
  const size_t V = a->V, fb = V * sizeof(float), nref = (size_t)N * N * (N + 2);
  CKA(cudaMemcpyAsync(a->pstage, Phi0, nref * sizeof(double), cudaMemcpyHostToDevice, st));
  CKA(launch_pair_from_ref(a->pstage, a->pph[0], a->ppl[0], N, st));
  CKA(cudaMemcpyAsync(a->pstage, Pi0, nref * sizeof(double), cudaMemcpyHostToDevice, st));
  CKA(launch_pair_from_ref(a->pstage, a->pqh, a->pql, N, st));
  h->launches += 2;
  // The steps and the checkpoint copies depend only on the buffers and the
  // clock factors (the same for every forward from reset()): captured once as
  // a CUDA graph, replayed per forward.
  if (!a->pgraph_ok) {
    a->fk.clear();
    a->fd.clear();
    a->sfk.clear();
    AdjClock ck_{a->p.T0, a->p.dt * a->p.a, a->p.T0, a->p.T0, 0.0, 0.0, a->p.T0, a->p.H0, a->p.expanding != 0};
    if (ck_.ex) ck_.tc = (sqrt(1. + 2. * ck_.H0 * ck_.tau) - 1.) / ck_.H0;  // phn_reset's conformal time
    ck_.lmc = ck_.lfc = ck_.tc;
    int cur = 0;
    char *ck = (char *)a->ckpt;
    CKA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaMemcpyAsync(ck, a->pph[0], fb, cudaMemcpyDeviceToDevice, st);
    if (le == cudaSuccess) le = cudaMemcpyAsync(ck + fb, a->pqh, fb, cudaMemcpyDeviceToDevice, st);
    for (int s = 0; s < a->nseg && le == cudaSuccess; ++s) {
      for (int i = 0; i < a->every && le == cudaSuccess; ++i) {
        double fk, fd, sfk;
        ck_.step(fk, fd, sfk);
        a->fk.push_back(fk);
        a->fd.push_back(fd);
        a->sfk.push_back(sfk);
        le = launch_step_pair(step_consts(a, (int)a->sfk.size() - 1), fk, fd, a->pph[cur], a->ppl[cur], a->pqh,
                              a->pql, a->pph[1 - cur], a->ppl[1 - cur], st);
        cur = 1 - cur;
      }
      if (le == cudaSuccess)
        le = cudaMemcpyAsync(ck + (size_t)(s + 1) * 2 * fb, a->pph[cur], fb, cudaMemcpyDeviceToDevice, st);
      if (le == cudaSuccess)
        le = cudaMemcpyAsync(ck + (size_t)(s + 1) * 2 * fb + fb, a->pqh, fb, cudaMemcpyDeviceToDevice, st);
    }
    a->sf_fin = ck_.sf();
    if (le == cudaSuccess) le = launch_pair_to_f64(a->pph[cur], a->ppl[cur], a->pfin, N, st);
    if (le == cudaSuccess) le = launch_pair_to_f64(a->pqh, a->pql, a->pfin + V, N, st);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return cuda_error(le != cudaSuccess ? le : ce, "pair forward capture");
    }
    const cudaError_t ie = cudaGraphInstantiate(&a->pgraph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return cuda_error(ie, "cudaGraphInstantiate (pair forward)");
    a->pgraph_ok = true;
  }
  CKA(cudaEventRecord(a->ev0, st));
  CKA(cudaGraphLaunch(a->pgraph, st));
  h->launches += a->nsteps + 2;
  return objective<double>(a, a->pfin, a->pfin + V, st);
}

int phn_adjoint_forward(phn_adjoint *a, const double *Phi0, const double *Pi0, double *J) {
  if (!a || !Phi0 || !Pi0) return set_error(PHN_ERR_INVALID, "NULL argument");
  if (a->pair) {
    int r = forward_pair(a, Phi0, Pi0);
    if (r) return r;
    cudaStream_t st = a->fwd->stream;
    CKA(cudaEventRecord(a->ev1, st));
    CKA(cudaEventSynchronize(a->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a->ev0, a->ev1);
    a->fwd_ms = ms;
    a->mean = a->h_res[0];
    a->J = a->h_res[1];
    a->S = a->h_res[2];
    a->forward_done = true;
    if (J) *J = a->J;
    return PHN_OK;
  }
  phn_handle *h = a->fwd;
  int r = phn_upload(h, Phi0, Pi0);
  if (r) return r;
  r = phn_reset(h);
  if (r) return r;
  void *phi = nullptr, *pi = nullptr, *stv = nullptr;
  const size_t fb = a->V * a->elem;
  char *ck = (char *)a->ckpt;
  a->fk.clear();
  a->fd.clear();
  a->sfk.clear();
  phn_device_fields(h, &phi, &pi, &stv);
  cudaStream_t st = (cudaStream_t)stv;
  // an FP64 forward under an FP32 reverse sweep stores FP32 checkpoints
  const bool narrow = a->fwd_elem == 8 && a->elem == 4;
  auto store = [&](char *dst, const void *src) -> cudaError_t {
    if (!narrow) return cudaMemcpyAsync(dst, src, fb, cudaMemcpyDeviceToDevice, st);
    narrow_f64<<<152 * 4, 256, 0, st>>>((const double *)src, (float *)dst, a->V);
    h->launches++;
    return cudaGetLastError();
  };
  CKA(cudaEventRecord(a->ev0, st));
  CKA(store(ck, phi));
  CKA(store(ck + fb, pi));
  for (int s = 0; s < a->nseg; ++s) {
    // the factors the next `every` steps will use: the clock arithmetic of
    // dynamics.cpp:196-237, as the handle runs it
    AdjClock ck_{h->tau, h->dtau, h->last_mom, h->last_field, h->last_mom_c, h->last_field_c, h->tau_c,
                 a->p.H0, a->p.expanding != 0};
    for (int i = 0; i < a->every; ++i) {
      double fk, fd, sfk;
      ck_.step(fk, fd, sfk);
      a->fk.push_back(fk);
      a->fd.push_back(fd);
      a->sfk.push_back(sfk);
    }
    r = evolve_async(h, a->every);
    if (r) return r;
    phn_device_fields(h, &phi, &pi, &stv);
    CKA(store(ck + (size_t)(s + 1) * 2 * fb, phi));
    CKA(store(ck + (size_t)(s + 1) * 2 * fb + fb, pi));
  }
  a->sf_fin = h->sf;
  if (a->fwd_elem == 8)
    r = objective<double>(a, (const double *)phi, (const double *)pi, st);
  else
    r = objective<float>(a, (const float *)phi, (const float *)pi, st);
  if (r) return r;
  CKA(cudaEventRecord(a->ev1, st));
  CKA(cudaEventSynchronize(a->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a->ev0, a->ev1);
  a->fwd_ms = ms;
  a->mean = a->h_res[0];
  a->J = a->h_res[1];
  a->S = a->h_res[2];
  a->forward_done = true;
  if (J) *J = a->J;
  return PHN_OK;
}

// grads[0] = dJ/d(homogeneous phi shift) = sum_x dJ/dphi_0(x)
// grads[1] = dJ/dc6, c6 the phi^6 coefficient of V (theory 0: 1/(720 Kappa^2))
// grads[2] = dJ/dh (theory 1)
int phn_adjoint_backward(phn_adjoint *a, double *dPhi0, double *dPi0, double *grads) {
  if (!a) return set_error(PHN_ERR_INVALID, "NULL argument");
  if (!a->forward_done) return set_error(PHN_ERR_INVALID, "phn_adjoint_forward first");
  phn_handle *h = a->fwd;
  void *phi = nullptr, *pi = nullptr, *stv = nullptr;
  phn_device_fields(h, &phi, &pi, &stv);
  cudaStream_t st = (cudaStream_t)stv;
  const size_t fb = a->V * a->elem;
  const bool dbl = a->elem == 8;
  const bool x4 = !dbl && a->p.N % 4 == 0;
  const Grid gr = adjoint_grid(a->p.N, x4);
  const int nb = a->sum_blocks;
  // The sweep's launches depend only on the handle's buffers and the clock
  // factors (identical for every forward from reset()): they are captured
  // once as a CUDA graph, before the timed region, and replayed.
  if (!a->graph_ok) {
    CKA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int cur = 0;  // lphi[cur], lpi[cur] hold the adjoint
    char *ck = (char *)a->ckpt;
    int sbuf = 0;
    cudaError_t le = cudaSuccess;
    for (int s = a->nseg - 1; s >= 0 && le == cudaSuccess; --s) {
      // re-anchor: the segment's end state is its checkpoint
      const void *phi1 = ck + (size_t)(s + 1) * 2 * fb;
      const void *pi1 = ck + (size_t)(s + 1) * 2 * fb + fb;
      for (int i = a->every - 1; i >= 0 && le == cudaSuccess; --i) {
        const int n = s * a->every + i;
        void *phi0 = a->rphi[sbuf], *pi0 = a->rpi[sbuf];
        // step n's couplings and its coupling-gradient factors: the kick's
        // V' holds c6 / sf^2 and h sf^3 in the expanding box (1 when static)
        const Consts kn = step_consts(a, n);
        const double sfk = a->sfk[n], s6 = 1.0 / (sfk * sfk), sh = sfk * sfk * sfk;
        const double fkT = dbl ? a->fk[n] : (double)(float)a->fk[n];
        if (dbl)
          adjoint_step<double><<<gr.grid, dim3(ADJ_TX, ADJ_TY), 0, st>>>(
              (const double *)phi1, (const double *)pi1, (const double *)a->lphi[cur], (const double *)a->lpi[cur],
              (double *)phi0, (double *)pi0, (double *)a->lphi[1 - cur], (double *)a->lpi[1 - cur], kn,
              a->fk[n], a->fd[n], fkT * s6, fkT * sh, gr.cz, a->gs);
        else if (x4)
          (a->k.theory == 0 ? adjoint_step_x4<0> : adjoint_step_x4<1>)<<<gr.grid, dim3(ADJ_TX, ADJ_TY), 0, st>>>(
              (const float *)phi1, (const float *)pi1, (const float *)a->lphi[cur], (const float *)a->lpi[cur],
              (float *)phi0, (float *)pi0, (float *)a->lphi[1 - cur], (float *)a->lpi[1 - cur], kn,
              (float)a->fk[n], (float)a->fd[n], (float)(fkT * s6), (float)(fkT * sh), gr.cz, a->gs);
        else
          adjoint_step<float><<<gr.grid, dim3(ADJ_TX, ADJ_TY), 0, st>>>(
              (const float *)phi1, (const float *)pi1, (const float *)a->lphi[cur], (const float *)a->lpi[cur],
              (float *)phi0, (float *)pi0, (float *)a->lphi[1 - cur], (float *)a->lpi[1 - cur], kn,
              (float)a->fk[n], (float)a->fd[n], fkT * s6, fkT * sh, gr.cz, a->gs);
        le = cudaGetLastError();
        cur = 1 - cur;
        phi1 = phi0;
        pi1 = pi0;
        sbuf = 1 - sbuf;
      }
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return cuda_error(le != cudaSuccess ? le : ce, "reverse sweep capture");
    }
    const cudaError_t ie = cudaGraphInstantiate(&a->sweep, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return cuda_error(ie, "cudaGraphInstantiate (reverse sweep)");
    a->graph_ok = true;
    a->final_cur = cur;
  }
  // timed: the seed at the final state and the reverse sweep
  CKA(cudaEventRecord(a->ev0, st));
  gs_zero<<<64, 256, 0, st>>>(a->gs, (size_t)gr.nblocks * ADJ_NG);
  // adjoint of the objective, with the direct dependence of rho on the couplings
  // (on the forward's final state: FP64 when the forward ran in FP64, the
  // pair state widened to FP64 when it ran in pairs)
  const DivN dn = make_divn((unsigned)a->k.N);
  const Consts kf = final_consts(a);
  if (dbl)
    obj_adjoint_init<double, double><<<nb, OBJ_THREADS, 0, st>>>((const double *)phi, (const double *)pi, a->g, kf, dn,
                                                                 (double *)a->lphi[0], (double *)a->lpi[0], a->sums,
                                                                 nb);
  else if (a->pair)
    obj_adjoint_init<double, float><<<nb, OBJ_THREADS, 0, st>>>(a->pfin, a->pfin + a->V, a->g, kf, dn,
                                                                (float *)a->lphi[0], (float *)a->lpi[0], a->sums, nb);
  else if (a->fwd_elem == 8)
    obj_adjoint_init<double, float><<<nb, OBJ_THREADS, 0, st>>>((const double *)phi, (const double *)pi, a->g, kf, dn,
                                                                (float *)a->lphi[0], (float *)a->lpi[0], a->sums, nb);
  else
    obj_adjoint_init<float, float><<<nb, OBJ_THREADS, 0, st>>>((const float *)phi, (const float *)pi, a->g, kf, dn,
                                                               (float *)a->lphi[0], (float *)a->lpi[0], a->sums, nb);
  CKA(cudaGetLastError());
  CKA(cudaGraphLaunch(a->sweep, st));
  h->launches += a->nsteps + 2;
  const int cur = a->final_cur;
  CKA(cudaEventRecord(a->ev1, st));
  CKA(cudaEventSynchronize(a->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a->ev0, a->ev1);
  a->bwd_ms = ms;
  // gradient slots and direct coupling terms, fixed order
  std::vector<double> gsh((size_t)gr.nblocks * ADJ_NG), dsh(2 * (size_t)nb);
  CKA(cudaMemcpy(gsh.data(), a->gs, gsh.size() * sizeof(double), cudaMemcpyDeviceToHost));
  CKA(cudaMemcpy(dsh.data(), a->sums, dsh.size() * sizeof(double), cudaMemcpyDeviceToHost));
  double g_c6 = 0.0, g_h = 0.0, direct_c6 = 0.0, direct_h = 0.0;
  for (int b = 0; b < gr.nblocks; ++b) {
    g_c6 += gsh[(size_t)b * ADJ_NG + 0];
    g_h += gsh[(size_t)b * ADJ_NG + 1];
  }
  for (int b = 0; b < nb; ++b) {
    direct_c6 += dsh[b];
    direct_h += dsh[nb + b];
  }
  // fields: lam_phi(0), lam_pi(0) in the reference layout, through the
  // handle's upload/download staging buffer
  const int N = a->p.N;
  // the reference-layout staging buffer: the handle's (allocated by its
  // upload) or, for a forward in pairs, which never uploads through the
  // handle, the pair forward's own
  double *ref = a->pair ? a->pstage : h->d_ref;
  if (!ref) return set_error(PHN_ERR_INVALID, "adjoint: no staging buffer (no forward upload)");
  const size_t slab = (size_t)N * N, nref = slab * (N + 2);
  double sum_lphi = 0.0;
  std::vector<double> tmp;
  if (dPhi0 || grads) {
    CKA(launch_to_ref(a->lphi[cur], ref, a->p.precision, N, 1, st));
    double *dst = dPhi0;
    if (!dst) {
      tmp.resize(nref);
      dst = tmp.data();
    }
    CKA(cudaMemcpyAsync(dst, ref, nref * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKA(cudaStreamSynchronize(st));
    for (size_t i = slab; i < slab * (N + 1); ++i) sum_lphi += dst[i];
  }
  if (dPi0) {
    CKA(launch_to_ref(a->lpi[cur], ref, a->p.precision, N, 1, st));
    CKA(cudaMemcpyAsync(dPi0 + slab, ref + slab, slab * N * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKA(cudaStreamSynchronize(st));
  }
  if (grads) {
    // J's own coupling terms: the final state's V holds c6 / sf^2 and h sf^3
    // in the expanding box
    const double sf = a->p.expanding ? a->sf_fin : 1.0;
    grads[0] = sum_lphi;
    grads[1] = g_c6 + (a->p.expanding ? direct_c6 / (sf * sf) : direct_c6);
    grads[2] = g_h + (a->p.expanding ? direct_h * (sf * sf * sf) : direct_h);
  }
  return PHN_OK;
}

int phn_adjoint_set_forward_precision(phn_adjoint *a, int precision) {
  if (!a) return set_error(PHN_ERR_INVALID, "NULL argument");
  const int cur = a->pair ? PHN_FP32_PAIR : (a->fwd_elem == 8 ? PHN_FP64 : PHN_FP32);
  if (precision == cur) return PHN_OK;
  if (a->p.precision != PHN_FP32 ||
      (precision != PHN_FP64 && precision != PHN_FP32 && precision != PHN_FP32_PAIR))
    return set_error(PHN_ERR_UNSUPPORTED, "forward precision: FP64, FP32 or FP32 pairs under an FP32 adjoint");
  if (precision == PHN_FP32_PAIR) {
    // the pair forward keeps the FP32 internal handle (its stream) and adds
    // its own buffers
    if (a->fwd_elem == 8) {
      const int r = phn_adjoint_set_forward_precision(a, PHN_FP32);
      if (r) return r;
    }
    if (!a->pqh) {
      const size_t fb = a->V * sizeof(float);
      const size_t nref = (size_t)a->p.N * a->p.N * (a->p.N + 2);
      cudaError_t e = cudaSuccess;
      for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaMalloc(&a->pph[i], fb);
        if (e == cudaSuccess) e = cudaMalloc(&a->ppl[i], fb);
      }
      if (e == cudaSuccess) e = cudaMalloc(&a->pqh, fb);
      if (e == cudaSuccess) e = cudaMalloc(&a->pql, fb);
      if (e == cudaSuccess) e = cudaMalloc(&a->pfin, 2 * a->V * sizeof(double));
      if (e == cudaSuccess) e = cudaMalloc(&a->pstage, nref * sizeof(double));
      if (e != cudaSuccess) return cuda_error(e, "pair forward buffers");
    }
    a->pair = true;
    a->forward_done = false;
    return PHN_OK;
  }
  a->pair = false;
  if (precision == (a->fwd_elem == 8 ? PHN_FP64 : PHN_FP32)) {
    a->forward_done = false;
    return PHN_OK;
  }
  phn_params q = a->p;
  q.precision = precision;
  phn_handle *nh = nullptr;
  const int r = phn_create(&q, &nh);
  if (r) return r;
  phn_destroy(a->fwd);
  a->fwd = nh;
  a->fwd_elem = precision == PHN_FP64 ? 8 : 4;
  a->forward_done = false;
  return PHN_OK;
}

int phn_adjoint_info(const phn_adjoint *a, double *J, double *forward_ms, double *backward_ms) {
  if (!a) return set_error(PHN_ERR_INVALID, "NULL argument");
  if (J) *J = a->J;
  if (forward_ms) *forward_ms = a->fwd_ms;
  if (backward_ms) *backward_ms = a->bwd_ms;
  return PHN_OK;
}

}  // extern "C"
