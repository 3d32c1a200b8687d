// Fused leapfrog step: kick (7-point Laplacian + potential force), drift into
// the second phi buffer, and optionally the volume averages and extrema of the
// state the step starts from -- all in one pass over HBM.
//
// Replaces updateMomenta + updateFields + Communication::exchange
// (dynamics.cpp:52-194, comm.cpp:63-78) and, on observation steps,
// CalculateVolumeAverages + CalculateExtrema (fieldanalysis.cpp:319-699).
// The periodic halo is in-kernel modular indexing; the MPI reductions become a
// deterministic two-stage tree (warp shuffles + shared memory per block, then
// finalize_averages over the block records in a fixed order).
//
// Work decomposition: a block is 32 x-sites by 8 y-rows and marches a chunk of
// z-planes, carrying phi(z-1), phi(z), phi(z+1) in registers, so every plane
// of phi is fetched from HBM once per chunk; x/y neighbours hit L1/L2.
#include <math.h>

#include "kick.cuh"
#include "observe.cuh"
#include "phn_internal.h"

namespace phn {

// ----------------------------------------------------------- FP64 kernel
// Force of theories 2-5 (Nc = 1) in the reference's order (dynamics.cpp:
// 109-157; the expanding box's forms :116-163 with the couplings of
// at_scale_factor and the per-site divisions by sf); sin and pow are CUDA's,
// so theories 2, 3 and 5 agree with the reference to rounding, not bitwise.
template <int THEORY>
__device__ __forceinline__ double force_f64_ext(const Consts &k, double lap, double c, double l) {
  if (THEORY == 3 && k.expansion) {  // sin(phi / (sf sqrt(M))), no phi/|phi| factor
    const double t = __dmul_rn(k.m3, sin(div_by(k, c, k.sf_sqrtm, k.r_sf_sqrtm, k.l_sf_sqrtm)));
    return __dadd_rn(__dadd_rn(lap, -__dmul_rn(k.mmono, c)), -t);
  }
  if (THEORY == 2 || THEORY == 3) {
    const double s = __dsqrt_rn(l);
    const double arg = k.expansion ? div_by(k, div_by(k, s, k.sf, k.r_sf, k.l_sf), k.sqrt_m, k.r_sqrtm, k.l_sqrtm)
                                   : div_by(k, s, k.sqrt_m, k.r_sqrtm, k.l_sqrtm);
    const double t = __dmul_rn(__dmul_rn(k.m3, c / s), sin(arg));
    if (THEORY == 2) return __dadd_rn(lap, -t);
    return __dadd_rn(__dadd_rn(lap, -__dmul_rn(k.mmono, c)), -t);
  }
  if (THEORY == 4) {
    const double coef = __dadd_rn(__dadd_rn(k.mmM, -(__dmul_rn(k.g, c) / 2.)),
                                  __dmul_rn(k.lm, div_by_near(k, l, k.six_nc, k.r_six_nc)));
    return __dadd_rn(lap, -__dmul_rn(coef, c));
  }
  if (k.expansion)
    return __dadd_rn(lap, -__dmul_rn(__dmul_rn(k.msq_sf2, c),
                                     pow(__dadd_rn(1., div_by(k, div_by(k, div_by(k, l, k.msq, k.r_msq, k.l_msq), k.sf, k.r_sf, k.l_sf),
                                                              k.sf, k.r_sf, k.l_sf)),
                                         k.p_mono - 1)));
  return __dadd_rn(lap, -__dmul_rn(__dmul_rn(k.msq, c), pow(__dadd_rn(1., div_by(k, l, k.msq, k.r_msq, k.l_msq)), k.p_mono - 1)));
}

// The kick and drift use explicit round-to-nearest intrinsics and IEEE
// division in the reference's operation order (dynamics.cpp:80-84,96-100,183),
// so every site value is bit-identical to the reference's FP64 build.
template <int NC, int THEORY, int MODE>
__global__ void __launch_bounds__(THREADS) step_f64(const double *__restrict__ phi, double *__restrict__ phi_out,
                                                    double *__restrict__ pi, const Consts k, const StepF s,
                                                    const int cz, double *__restrict__ partials) {
  const int N = k.N;
  const int x = blockIdx.x * TX + threadIdx.x;
  const int y = blockIdx.y * TY + threadIdx.y;
  const int z0 = blockIdx.z * cz;
  const int z1 = min(z0 + cz, N);
  const size_t NN = (size_t)N * N, V = NN * N;
  Acc acc;
  if (MODE != MODE_STEP) acc.init();
  if (x < N && y < N && z0 < z1) {
    const int xp = (x + 1 == N) ? 0 : x + 1, xm = (x == 0) ? N - 1 : x - 1;
    const int yp = (y + 1 == N) ? 0 : y + 1, ym = (y == 0) ? N - 1 : y - 1;
    double cm[NC], c[NC], cp[NC];
    const size_t col = (size_t)y * N + x;
    const int zm0 = (z0 == 0) ? N - 1 : z0 - 1;
#pragma unroll
    for (int a = 0; a < NC; ++a) {
      cm[a] = phi[a * V + zm0 * NN + col];
      c[a] = phi[a * V + z0 * NN + col];
    }
    for (int z = z0; z < z1; ++z) {
      const int zn = (z + 1 == N) ? 0 : z + 1;
      const size_t pl = (size_t)z * NN;
      double fxp[NC], fxm[NC], fyp[NC], fym[NC], p[NC];
#pragma unroll
      for (int a = 0; a < NC; ++a) {
        cp[a] = phi[a * V + zn * NN + col];
        fxp[a] = phi[a * V + pl + (size_t)y * N + xp];
        fxm[a] = phi[a * V + pl + (size_t)y * N + xm];
        fyp[a] = phi[a * V + pl + (size_t)yp * N + x];
        fym[a] = phi[a * V + pl + (size_t)ym * N + x];
        p[a] = pi[a * V + pl + col];
      }
      if (MODE != MODE_STEP)
        observe<NC, THEORY>(acc, k, c, p, fxp, fyp, cp, (long long)NC * (long long)(col + (size_t)(z + 1) * NN));
      if (MODE != MODE_OBS) {
        double l = 0.0;
#pragma unroll
        for (int a = 0; a < NC; ++a) l = __dadd_rn(l, __dmul_rn(c[a], c[a]));
        double coef = __dadd_rn(k.mmM, __dmul_rn(k.lm, div_by_near(k, l, k.six_nc, k.r_six_nc)));
        if (THEORY == 0) {
          double r = div_by(k, l, k.kappa, k.r_kappa, k.l_kappa);
          if (k.expansion) r = div_by(k, r, k.sf, k.r_sf, k.l_sf);  // sqr(locPhiSqr / Kappa / scale_factor) (dynamics.cpp:90)
          coef = __dadd_rn(coef, div_by_near(k, __dmul_rn(r, r), k.c120, k.r_c120));
        }
#pragma unroll
        for (int a = 0; a < NC; ++a) {
          const double sum = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(fxp[a], fxm[a]), fyp[a]), fym[a]), cp[a]), cm[a]);
          const double lap = div_a2(k, __dadd_rn(sum, -__dmul_rn(6.0, c[a])));
          double f = lap;
          if (THEORY <= 1) {
            if (THEORY == 1 && a == 0) f = __dadd_rn(f, -k.h);
            f = __dadd_rn(f, -__dmul_rn(coef, c[a]));
          } else {
            f = force_f64_ext<THEORY>(k, lap, c[a], l);
          }
          const double pn = __dadd_rn(p[a], __dmul_rn(f, s.fk));
          pi[a * V + pl + col] = pn;
          phi_out[a * V + pl + col] = __dadd_rn(c[a], __dmul_rn(pn, s.fd));
        }
      }
#pragma unroll
      for (int a = 0; a < NC; ++a) {
        cm[a] = c[a];
        c[a] = cp[a];
      }
    }
  }
  if (MODE != MODE_STEP) block_store(acc, partials);
}

// ----------------------------------------------------------- FP32 kernel
template <int NC, int THEORY, int MODE>
__global__ void __launch_bounds__(THREADS) step_f32(const float *__restrict__ phi, float *__restrict__ phi_out,
                                                    float *__restrict__ pi, const Consts k, const float fk,
                                                    const float fd, const int cz, double *__restrict__ partials) {
  const int N = k.N;
  const int x = blockIdx.x * TX + threadIdx.x;
  const int y = blockIdx.y * TY + threadIdx.y;
  const int z0 = blockIdx.z * cz;
  const int z1 = min(z0 + cz, N);
  const size_t NN = (size_t)N * N, V = NN * N;
  AccF accf;
  if (MODE != MODE_STEP) accf.init();
  if (x < N && y < N && z0 < z1) {
    const int xp = (x + 1 == N) ? 0 : x + 1, xm = (x == 0) ? N - 1 : x - 1;
    const int yp = (y + 1 == N) ? 0 : y + 1, ym = (y == 0) ? N - 1 : y - 1;
    float cm[NC], c[NC], cp[NC];
    const size_t col = (size_t)y * N + x;
    const int zm0 = (z0 == 0) ? N - 1 : z0 - 1;
#pragma unroll
    for (int a = 0; a < NC; ++a) {
      cm[a] = __ldg(phi + a * V + zm0 * NN + col);
      c[a] = __ldg(phi + a * V + z0 * NN + col);
    }
    for (int z = z0; z < z1; ++z) {
      const int zn = (z + 1 == N) ? 0 : z + 1;
      const size_t pl = (size_t)z * NN;
      float fxp[NC], fxm[NC], fyp[NC], fym[NC], p[NC];
#pragma unroll
      for (int a = 0; a < NC; ++a) {
        cp[a] = __ldg(phi + a * V + zn * NN + col);
        fxp[a] = __ldg(phi + a * V + pl + (size_t)y * N + xp);
        fxm[a] = __ldg(phi + a * V + pl + (size_t)y * N + xm);
        fyp[a] = __ldg(phi + a * V + pl + (size_t)yp * N + x);
        fym[a] = __ldg(phi + a * V + pl + (size_t)ym * N + x);
        p[a] = pi[a * V + pl + col];
      }
      if (MODE != MODE_STEP)
        observe_f32<NC, THEORY>(accf, k, c, p, fxp, fyp, cp, (long long)NC * (long long)(col + (size_t)(z + 1) * NN));
      if (MODE != MODE_OBS) {
        float l = 0.f;
#pragma unroll
        for (int a = 0; a < NC; ++a) l = fmaf(c[a], c[a], l);
        float coef = fmaf(l, k.c4_f, k.mmM_f);
        if (THEORY == 0) coef = fmaf(__fmul_rn(l, l), k.c6_f, coef);
#pragma unroll
        for (int a = 0; a < NC; ++a) {
          // the shared neighbour-difference Laplacian: the TMA kernel computes the same bits
          const float lap = lap_diff_f32(c[a], fxm[a], fxp[a], fym[a], fyp[a], cm[a], cp[a], k.inv_a2_f);
          float f;
          if (NC == 1 || THEORY >= 2) {  // theories 2-5 take the component sum l as well
            f = force_f32<THEORY>(k, lap, c[a], l);
          } else {
            f = fmaf(-coef, c[a], lap);
            if (THEORY == 1 && a == 0) f = __fsub_rn(f, k.h_f);
          }
          const float pn = fmaf(fk, f, p[a]);
          pi[a * V + pl + col] = pn;
          phi_out[a * V + pl + col] = fmaf(fd, pn, c[a]);
        }
      }
#pragma unroll
      for (int a = 0; a < NC; ++a) {
        cm[a] = c[a];
        c[a] = cp[a];
      }
    }
  }
  if (MODE != MODE_STEP) {
    Acc acc;
    accf.to_double(acc);
    block_store(acc, partials);
  }
}

// ------------------------------------------------ compensated FP32 kernel
// phi, pi in FP32 with FP32 compensation terms (Kahan): the represented
// value is hi - comp.  Kick and drift add their increments with Kahan's
// update, so the rounding error of each addition is carried instead of lost.
// comp arrays are per site (no stencil reads), updated in place.
template <int NC, int THEORY, int MODE>
__global__ void __launch_bounds__(THREADS) step_kahan(const float *__restrict__ phi, float *__restrict__ phi_out,
                                                      float *__restrict__ cphi, float *__restrict__ pi,
                                                      float *__restrict__ cpi, const Consts k, const float fk,
                                                      const float fd, const int cz, double *__restrict__ partials) {
  const int N = k.N;
  const int x = blockIdx.x * TX + threadIdx.x;
  const int y = blockIdx.y * TY + threadIdx.y;
  const int z0 = blockIdx.z * cz;
  const int z1 = min(z0 + cz, N);
  const size_t NN = (size_t)N * N, V = NN * N;
  AccF accf;
  if (MODE != MODE_STEP) accf.init();
  if (x < N && y < N && z0 < z1) {
    const int xp = (x + 1 == N) ? 0 : x + 1, xm = (x == 0) ? N - 1 : x - 1;
    const int yp = (y + 1 == N) ? 0 : y + 1, ym = (y == 0) ? N - 1 : y - 1;
    float cm[NC], c[NC], cp[NC];
    const size_t col = (size_t)y * N + x;
    const int zm0 = (z0 == 0) ? N - 1 : z0 - 1;
#pragma unroll
    for (int a = 0; a < NC; ++a) {
      cm[a] = __ldg(phi + a * V + zm0 * NN + col);
      c[a] = __ldg(phi + a * V + z0 * NN + col);
    }
    for (int z = z0; z < z1; ++z) {
      const int zn = (z + 1 == N) ? 0 : z + 1;
      const size_t pl = (size_t)z * NN;
      float fxp[NC], fxm[NC], fyp[NC], fym[NC], p[NC], ec[NC], ep[NC];
#pragma unroll
      for (int a = 0; a < NC; ++a) {
        cp[a] = __ldg(phi + a * V + zn * NN + col);
        fxp[a] = __ldg(phi + a * V + pl + (size_t)y * N + xp);
        fxm[a] = __ldg(phi + a * V + pl + (size_t)y * N + xm);
        fyp[a] = __ldg(phi + a * V + pl + (size_t)yp * N + x);
        fym[a] = __ldg(phi + a * V + pl + (size_t)ym * N + x);
        p[a] = pi[a * V + pl + col];
        ec[a] = cphi[a * V + pl + col];
        ep[a] = cpi[a * V + pl + col];
      }
      if (MODE != MODE_STEP) {
        // observables of the represented values hi - comp (neighbours: hi only)
        float cr[NC], pr[NC];
#pragma unroll
        for (int a = 0; a < NC; ++a) {
          cr[a] = __fsub_rn(c[a], ec[a]);
          pr[a] = __fsub_rn(p[a], ep[a]);
        }
        observe_f32<NC, THEORY>(accf, k, cr, pr, fxp, fyp, cp, (long long)NC * (long long)(col + (size_t)(z + 1) * NN));
      }
      if (MODE != MODE_OBS) {
        float l = 0.f;
#pragma unroll
        for (int a = 0; a < NC; ++a) l = fmaf(c[a], c[a], l);
        float coef = fmaf(l, k.c4_f, k.mmM_f);
        if (THEORY == 0) coef = fmaf(__fmul_rn(l, l), k.c6_f, coef);
#pragma unroll
        for (int a = 0; a < NC; ++a) {
          // the shared neighbour-difference Laplacian: the TMA kernel computes the same bits
          const float lap = lap_diff_f32(c[a], fxm[a], fxp[a], fym[a], fyp[a], cm[a], cp[a], k.inv_a2_f);
          float f;
          if (NC == 1 || THEORY >= 2) {  // theories 2-5 take the component sum l as well
            f = force_f32<THEORY>(k, lap, c[a], l);
          } else {
            f = fmaf(-coef, c[a], lap);
            if (THEORY == 1 && a == 0) f = __fsub_rn(f, k.h_f);
          }
          // kick: pi += fk * f  (Kahan)
          const float yk = __fsub_rn(__fmul_rn(fk, f), ep[a]);
          const float tk = __fadd_rn(p[a], yk);
          const float ek = __fsub_rn(__fsub_rn(tk, p[a]), yk);
          // drift: phi += fd * pi_new  (Kahan); the increment uses the
          // represented momentum tk - ek
          const float yd = __fsub_rn(__fmul_rn(fd, __fsub_rn(tk, ek)), ec[a]);
          const float td = __fadd_rn(c[a], yd);
          const float ed = __fsub_rn(__fsub_rn(td, c[a]), yd);
          pi[a * V + pl + col] = tk;
          cpi[a * V + pl + col] = ek;
          phi_out[a * V + pl + col] = td;
          cphi[a * V + pl + col] = ed;
        }
      }
#pragma unroll
      for (int a = 0; a < NC; ++a) {
        cm[a] = c[a];
        c[a] = cp[a];
      }
    }
  }
  if (MODE != MODE_STEP) {
    Acc acc;
    accf.to_double(acc);
    block_store(acc, partials);
  }
}

// ----------------------------------------------------------- finalize
__global__ void __launch_bounds__(FIN_THREADS) finalize_averages(const double *__restrict__ partials, int nblocks,
                                                                 const Consts k, phn_averages *__restrict__ out) {
  fold_records(partials, 0, nblocks, k, out);
}

// First level of a two-level fold: block g folds records [g FIN_GROUP,
// (g+1) FIN_GROUP) into group record g.
__global__ void __launch_bounds__(FIN_THREADS) fold_groups(const double *__restrict__ partials, int nblocks,
                                                           double *__restrict__ groups) {
  __shared__ double sh[FIN_THREADS][REC];
  const int b0 = blockIdx.x * FIN_GROUP, b1 = min(nblocks, b0 + FIN_GROUP);
  fold_acc(partials, b0, b1, sh);
  if (threadIdx.x == 0)
    for (int j = 0; j < REC; ++j) groups[(size_t)blockIdx.x * REC + j] = sh[0][j];
}

// ----------------------------------------------------------- launchers
Grid lattice_grid(int N) {
  Grid g;
  g.block = dim3(TX, TY, 1);
  const int gx = (N + TX - 1) / TX, gy = (N + TY - 1) / TY;
  int cz;
  if (N >= 256)
    cz = 16;
  else if (N >= 128)
    cz = 8;
  else {
    // small lattices: enough blocks to fill the GPU, planes per block >= 1
    const long long cols = (long long)gx * gy;
    const long long want = 152LL * 8;
    const long long gz = (want + cols - 1) / cols;
    cz = (int)((N + gz - 1) / gz);
    if (cz < 1) cz = 1;
  }
  const int gz = (N + cz - 1) / cz;
  g.grid = dim3(gx, gy, gz);
  g.cz = cz;
  g.nblocks = gx * gy * gz;
  return g;
}

#define PHN_DISPATCH_NC(NCV, ...)                              \
  switch (NCV) {                                               \
    case 1: { constexpr int NC_ = 1; __VA_ARGS__; } break;     \
    case 2: { constexpr int NC_ = 2; __VA_ARGS__; } break;     \
    case 3: { constexpr int NC_ = 3; __VA_ARGS__; } break;     \
    case 4: { constexpr int NC_ = 4; __VA_ARGS__; } break;     \
    default: return cudaErrorInvalidValue;                     \
  }

#define PHN_DISPATCH_TH(THV, ...)                              \
  if ((THV) == 0) { constexpr int TH_ = 0; __VA_ARGS__; }      \
  else { constexpr int TH_ = 1; __VA_ARGS__; }

// Every theory for every component count.
#define PHN_DISPATCH_TH6(THV, ...)                                                 \
  if ((THV) == 0) { constexpr int TH_ = 0; __VA_ARGS__; }                          \
  else if ((THV) == 1) { constexpr int TH_ = 1; __VA_ARGS__; }                     \
  else if ((THV) == 2) { constexpr int TH_ = 2; __VA_ARGS__; }                     \
  else if ((THV) == 3) { constexpr int TH_ = 3; __VA_ARGS__; }                     \
  else if ((THV) == 4) { constexpr int TH_ = 4; __VA_ARGS__; }                     \
  else { constexpr int TH_ = 5; __VA_ARGS__; }

#define PHN_DISPATCH_NC_TH(NCV, THV, ...) PHN_DISPATCH_NC(NCV, PHN_DISPATCH_TH6(THV, __VA_ARGS__))

#define PHN_DISPATCH_MODE(MV, ...)                             \
  if ((MV) == MODE_STEP) { constexpr int MD_ = MODE_STEP; __VA_ARGS__; }          \
  else if ((MV) == MODE_STEP_OBS) { constexpr int MD_ = MODE_STEP_OBS; __VA_ARGS__; } \
  else { constexpr int MD_ = MODE_OBS; __VA_ARGS__; }

cudaError_t launch_step_f64(const Consts &k, const Grid &g, int mode, const double *phi, double *phi_out,
                            double *pi, StepF s, double *partials, cudaStream_t st) {
  PHN_DISPATCH_NC_TH(k.Nc, k.theory, PHN_DISPATCH_MODE(mode,
      step_f64<NC_, TH_, MD_><<<g.grid, g.block, 0, st>>>(phi, phi_out, pi, k, s, g.cz, partials)));
  return cudaGetLastError();
}

cudaError_t launch_step_f32(const Consts &k, const Grid &g, int mode, const float *phi, float *phi_out,
                            float *pi, StepF s, double *partials, cudaStream_t st) {
  const float fk = (float)s.fk, fd = (float)s.fd;
  PHN_DISPATCH_NC_TH(k.Nc, k.theory, PHN_DISPATCH_MODE(mode,
      step_f32<NC_, TH_, MD_><<<g.grid, g.block, 0, st>>>(phi, phi_out, pi, k, fk, fd, g.cz, partials)));
  return cudaGetLastError();
}

cudaError_t launch_step_kahan(const Consts &k, const Grid &g, int mode, const float *phi, float *phi_out,
                              const float *cphi, float *cphi_out, float *pi, float *cpi, StepF s,
                              double *partials, cudaStream_t st) {
  (void)cphi;
  const float fk = (float)s.fk, fd = (float)s.fd;
  PHN_DISPATCH_NC_TH(k.Nc, k.theory, PHN_DISPATCH_MODE(mode,
      step_kahan<NC_, TH_, MD_><<<g.grid, g.block, 0, st>>>(phi, phi_out, cphi_out, pi, cpi, k, fk, fd, g.cz,
                                                            partials)));
  return cudaGetLastError();
}

// Many records (one block per item at 512^3: 16384) fold in two levels, so
// that one block does not walk them all: groups of FIN_GROUP records into
// groups[], then those.  Both levels keep a fixed order.
cudaError_t launch_finalize(const Consts &k, const double *partials, int nblocks, phn_averages *out,
                            cudaStream_t st, double *groups, int groups_cap) {
  const int ng = (nblocks + FIN_GROUP - 1) / FIN_GROUP;
  if (groups && nblocks > 4 * FIN_GROUP && ng <= groups_cap) {
    fold_groups<<<ng, FIN_THREADS, 0, st>>>(partials, nblocks, groups);
    finalize_averages<<<1, FIN_THREADS, 0, st>>>(groups, ng, k, out);
  } else {
    finalize_averages<<<1, FIN_THREADS, 0, st>>>(partials, nblocks, k, out);
  }
  return cudaGetLastError();
}

}  // namespace phn
