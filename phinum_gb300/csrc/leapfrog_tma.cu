// TMA-pipelined leapfrog step for FP32 fields, one component, N a multiple
// of 128 (the production path for the large lattices).
//
// Same arithmetic as step_f32 (leapfrog.cu) -- the kernels produce
// bit-identical fields -- with a different memory pipeline:
//   * a persistent grid (blocks = SMs x resident blocks); block b owns the
//     contiguous range [W*b/G, W*(b+1)/G) of the plane-tiles
//     w = tile*N + z, a tile being TY full lattice rows, so work is balanced
//     to one plane-tile and each block marches long runs of z;
//   * one producer lane issues 1-D bulk copies (cp.async.bulk, the TMA
//     engine) of each plane-tile into a ring of S shared-memory stages:
//     phi rows y0-1 .. y0+TY (y halo, periodic wrap as two copies) and, in
//     the PI_SMEM variants, the tile's pi rows, completing on the stage's
//     "full" mbarrier;
//   * TY consumer warps (one per row) read the stage, take x neighbours by
//     warp shuffles (a warp holds whole rows, so the periodic x wrap is a
//     shuffle too), keep phi(z-1), phi(z), phi(z+1) in registers, stream pi
//     (from the stage, or straight from HBM one plane ahead), write pi' and
//     phi' with 16-byte stores, then release the stage on its "empty"
//     mbarrier.
// HBM traffic per site: phi once plus the y halo ((TY+2)/TY, partly served by
// L2), pi once, pi' and phi' once: 16 B algorithmic.
//
// Variants (TY, S, PI_SMEM) trade halo re-reads against shared memory per
// block; phn_autotune times them on the live lattice and keeps the fastest.
#include "kick.cuh"
#include "observe.cuh"
#include "phn_internal.h"
#include "tma.cuh"

namespace phn {

// Kernel configurations (tile height TY, stages S, pi through shared memory)
// and variants = configuration x grid policy.  "aligned" grids use
// G = (N/TY) * m blocks with m | N, so a block's range of plane-tiles is
// N/m planes of one tile and the blocks working on vertically adjacent tiles
// are at the same z at the same time: the y-halo rows one block loads are the
// rows its neighbours loaded moments earlier, still in L2.
struct TmaConfig {
  int ty, stages;
  bool pi_smem;
};
constexpr TmaConfig kTmaConfigs[] = {{4, 4, true}, {8, 4, false}, {8, 5, false}, {4, 6, false}};
struct TmaVariantDef {
  int config;
  bool aligned;
};
constexpr TmaVariantDef kTmaVariants[] = {{0, false}, {1, false}, {2, false}, {3, false},
                                          {1, true},  {0, true},  {2, true}};
constexpr int kNumTmaVariants = 7;

template <int K, int TY, int S, bool PI_SMEM>
struct TmaShape {
  static constexpr int N = K * 128;
  static constexpr int PHI_ROWS = TY + 2;
  static constexpr int STAGE_FLOATS = (PHI_ROWS + (PI_SMEM ? TY : 0)) * N;
  static constexpr uint32_t PHI_BYTES = PHI_ROWS * N * 4;
  static constexpr uint32_t PI_BYTES = TY * N * 4;
  static constexpr int THREADS = (TY + 1) * 32;
  static constexpr size_t SMEM = 128 + (size_t)S * STAGE_FLOATS * sizeof(float);
};

__device__ __forceinline__ float get(const float4 &v, int e) {
  return e == 0 ? v.x : (e == 1 ? v.y : (e == 2 ? v.z : v.w));
}

template <int K, int TY, int S, bool PI_SMEM, int THEORY, bool OBS>
__global__ void __launch_bounds__((TY + 1) * 32) step_f32_tma(const float *__restrict__ phi,
                                                              float *__restrict__ phi_out, float *__restrict__ pi,
                                                              const Consts k, const float fk, const float fd,
                                                              double *__restrict__ partials, int *__restrict__ err) {
  using Sh = TmaShape<K, TY, S, PI_SMEM>;
  constexpr int N = Sh::N;
  constexpr long long NN = (long long)N * N;
  constexpr long long W = (long long)(N / TY) * N;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int abort_flag;
  uint64_t *bars = (uint64_t *)smem;  // full[S], empty[S]
  float *stages = (float *)(smem + 128);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long w0 = W * blockIdx.x / gridDim.x, w1 = W * (blockIdx.x + 1) / gridDim.x;
  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < S; ++s) {
      mbar_init(smem_u32(&bars[s]), 1);
      mbar_init(smem_u32(&bars[S + s]), TY);
    }
    mbar_fence_init();
  }
  __syncthreads();

  AccF accf;
  if (OBS) accf.init();

  if (warp == TY) {
    // ---------------------------------------------------------- producer
    if (lane == 0) {
      long long L = 0;
      bool ok = true;
      for (long long w = w0; w < w1 && ok;) {
        const int t = (int)(w / N), za = (int)(w % N);
        const long long wend = min(w1, (long long)(t + 1) * N);
        const int zb = za + (int)(wend - w);
        const int y0 = t * TY;
        for (int j = -1; j <= zb - za && ok; ++j) {
          const int z = (za + j + N) % N;
          const bool center = PI_SMEM && (j >= 0 && j < zb - za);
          const int s = (int)(L % S);
          const long long n = L / S;
          if (n > 0) {
            ok = mbar_wait(smem_u32(&bars[S + s]), (uint32_t)((n - 1) & 1), err, 1, &abort_flag);
            if (!ok) break;
          }
          const uint32_t full = smem_u32(&bars[s]);
          mbar_arrive_expect_tx(full, Sh::PHI_BYTES + (center ? Sh::PI_BYTES : 0u));
          const uint32_t dst = smem_u32(stages + (size_t)s * Sh::STAGE_FLOATS);
          const float *plane = phi + (long long)z * NN;
          constexpr uint32_t ROWB = N * 4;
          if (y0 == 0) {
            bulk_g2s(dst, plane + (long long)(N - 1) * N, ROWB, full);
            bulk_g2s(dst + ROWB, plane, ROWB * (TY + 1), full);
          } else if (y0 + TY == N) {
            bulk_g2s(dst, plane + (long long)(y0 - 1) * N, ROWB * (TY + 1), full);
            bulk_g2s(dst + ROWB * (TY + 1), plane, ROWB, full);
          } else {
            bulk_g2s(dst, plane + (long long)(y0 - 1) * N, ROWB * (TY + 2), full);
          }
          if (center) bulk_g2s(dst + Sh::PHI_BYTES, pi + (long long)z * NN + (long long)y0 * N, Sh::PI_BYTES, full);
          ++L;
        }
        w = wend;
      }
      if (!ok) {
        // drain: wait (bounded) until the copies already issued -- at most
        // the last S loads, one per stage -- have landed before exiting
        for (long long q = (L > S ? L - S : 0); q < L; ++q)
          mbar_wait(smem_u32(&bars[q % S]), (uint32_t)((q / S) & 1), nullptr, 0, nullptr);
      }
    }
  } else {
    // ---------------------------------------------------------- consumers
    long long L = 0;
    float4 cm[K], c[K], cp[K], pnx[K];
    const int r = warp;  // row within the tile
    bool ok = true;
    for (long long w = w0; w < w1 && ok;) {
      const int t = (int)(w / N), za = (int)(w % N);
      const long long wend = min(w1, (long long)(t + 1) * N);
      const int zb = za + (int)(wend - w);
      const int y = t * TY + r;
      if (!PI_SMEM) {
#pragma unroll
        for (int q = 0; q < K; ++q)
          pnx[q] = __ldcs((const float4 *)(pi + (long long)za * NN + (long long)y * N + 128 * q + 4 * lane));
      }
      // plane za-1: its centre row becomes phi(z-1)
      {
        const int s = (int)(L % S);
        ok = mbar_wait(smem_u32(&bars[s]), (uint32_t)((L / S) & 1), err, 2, &abort_flag);
        if (!ok) break;
        const float *row = stages + (size_t)s * Sh::STAGE_FLOATS + (r + 1) * N;
#pragma unroll
        for (int q = 0; q < K; ++q) cm[q] = *(const float4 *)(row + 128 * q + 4 * lane);
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&bars[S + s]));
        ++L;
      }
      // plane za: phi(z)
      {
        const int s = (int)(L % S);
        ok = mbar_wait(smem_u32(&bars[s]), (uint32_t)((L / S) & 1), err, 2, &abort_flag);
        if (!ok) break;
        const float *row = stages + (size_t)s * Sh::STAGE_FLOATS + (r + 1) * N;
#pragma unroll
        for (int q = 0; q < K; ++q) c[q] = *(const float4 *)(row + 128 * q + 4 * lane);
        ++L;
      }
      for (int z = za; z < zb; ++z) {
        const int sz = (int)((L - 1) % S);
        const int s1 = (int)(L % S);
        const long long gz = (long long)z * NN + (long long)y * N;
        float4 pcur[K];
#pragma unroll
        for (int q = 0; q < K; ++q) pcur[q] = pnx[q];
        if (!PI_SMEM && z + 1 < zb) {
#pragma unroll
          for (int q = 0; q < K; ++q) pnx[q] = __ldcs((const float4 *)(pi + gz + NN + 128 * q + 4 * lane));
        }
        ok = mbar_wait(smem_u32(&bars[s1]), (uint32_t)((L / S) & 1), err, 2, &abort_flag);
        if (!ok) break;
        const float *nrow = stages + (size_t)s1 * Sh::STAGE_FLOATS + (r + 1) * N;
#pragma unroll
        for (int q = 0; q < K; ++q) cp[q] = *(const float4 *)(nrow + 128 * q + 4 * lane);
        const float *st = stages + (size_t)sz * Sh::STAGE_FLOATS;
        PlaneF plane;
        if (OBS) plane.clear();
#pragma unroll
        for (int q = 0; q < K; ++q) {
          const int x0 = 128 * q + 4 * lane;
          const float4 ym = *(const float4 *)(st + r * N + x0);
          const float4 yp = *(const float4 *)(st + (r + 2) * N + x0);
          const float4 pv = PI_SMEM ? *(const float4 *)(st + (Sh::PHI_ROWS + r) * N + x0) : pcur[q];
          // x neighbours: within the lane, from lanes -+1, and across chunks at the warp edges
          float left = __shfl_up_sync(0xffffffffu, c[q].w, 1);
          const float lwrap = __shfl_sync(0xffffffffu, c[(q + K - 1) % K].w, 31);
          float right = __shfl_down_sync(0xffffffffu, c[q].x, 1);
          const float rwrap = __shfl_sync(0xffffffffu, c[(q + 1) % K].x, 0);
          if (lane == 0) left = lwrap;
          if (lane == 31) right = rwrap;
          float4 pn, fn;
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float cc = get(c[q], e);
            const float xm = e == 0 ? left : get(c[q], e - 1);
            const float xp = e == 3 ? right : get(c[q], e + 1);
            const float ymv = get(ym, e), ypv = get(yp, e), zm = get(cm[q], e), zp = get(cp[q], e);
            const float pp = get(pv, e);
            if (OBS) observe_site<THEORY>(plane, accf, k, cc, pp, xp, ypv, zp, gz + NN + x0 + e);
            float pnv, fnv;
            kick_drift_f32<THEORY>(k, fk, fd, cc, xm, xp, ymv, ypv, zm, zp, pp, pnv, fnv);
            if (e == 0) { pn.x = pnv; fn.x = fnv; }
            if (e == 1) { pn.y = pnv; fn.y = fnv; }
            if (e == 2) { pn.z = pnv; fn.z = fnv; }
            if (e == 3) { pn.w = pnv; fn.w = fnv; }
          }
          *(float4 *)(pi + gz + x0) = pn;
          *(float4 *)(phi_out + gz + x0) = fn;
        }
        if (OBS) flush_plane(accf, plane);
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&bars[S + sz]));
#pragma unroll
        for (int q = 0; q < K; ++q) {
          cm[q] = c[q];
          c[q] = cp[q];
        }
        ++L;
      }
      if (!ok) break;
      // release the stage of plane zb (used as phi(z+1) of the last plane)
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&bars[S + (int)((L - 1) % S)]));
      w = wend;
    }
  }
  if (OBS) {
    Acc acc;
    if (warp < TY)
      accf.to_double(acc);
    else
      acc.init();
    block_store_n(acc, partials, tid, TY + 1, blockIdx.x);
  }
}

// --------------------------------------------------------------- dispatch
template <int K, int TY, int S, bool PS>
struct TmaLaunch {
  using Sh = TmaShape<K, TY, S, PS>;
  template <int TH, bool OB>
  static const void *fn() {
    return (const void *)step_f32_tma<K, TY, S, PS, TH, OB>;
  }
  static cudaError_t prepare() {
    cudaError_t e;
    const void *fns[4] = {fn<0, false>(), fn<0, true>(), fn<1, false>(), fn<1, true>()};
    for (const void *f : fns)
      if ((e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Sh::SMEM)) != cudaSuccess)
        return e;
    return cudaSuccess;
  }
  static int occupancy() {
    int occ = 0;
    if (prepare() != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn<0, false>(), Sh::THREADS, Sh::SMEM) != cudaSuccess)
      return 0;
    return occ;
  }
  static cudaError_t launch(const Consts &k, bool obs, int grid, const float *phi, float *phi_out, float *pi,
                            float fk, float fd, double *partials, int *err, cudaStream_t st) {
    if (k.theory == 0) {
      if (obs)
        step_f32_tma<K, TY, S, PS, 0, true><<<grid, Sh::THREADS, Sh::SMEM, st>>>(phi, phi_out, pi, k, fk, fd, partials, err);
      else
        step_f32_tma<K, TY, S, PS, 0, false><<<grid, Sh::THREADS, Sh::SMEM, st>>>(phi, phi_out, pi, k, fk, fd, partials, err);
    } else {
      if (obs)
        step_f32_tma<K, TY, S, PS, 1, true><<<grid, Sh::THREADS, Sh::SMEM, st>>>(phi, phi_out, pi, k, fk, fd, partials, err);
      else
        step_f32_tma<K, TY, S, PS, 1, false><<<grid, Sh::THREADS, Sh::SMEM, st>>>(phi, phi_out, pi, k, fk, fd, partials, err);
    }
    return cudaGetLastError();
  }
};

// Calls F<K, TY, S, PI_SMEM>::... for the runtime (K, variant).
#define PHN_TMA_SWITCH(KV, CFG, EXPR_T, FAIL)                                   \
  switch ((KV) * 16 + (CFG)) {                                                  \
    case 1 * 16 + 0: { using T = TmaLaunch<1, 4, 4, true>; EXPR_T; }            \
    case 1 * 16 + 1: { using T = TmaLaunch<1, 8, 4, false>; EXPR_T; }           \
    case 1 * 16 + 2: { using T = TmaLaunch<1, 8, 5, false>; EXPR_T; }           \
    case 1 * 16 + 3: { using T = TmaLaunch<1, 4, 6, false>; EXPR_T; }           \
    case 2 * 16 + 0: { using T = TmaLaunch<2, 4, 4, true>; EXPR_T; }            \
    case 2 * 16 + 1: { using T = TmaLaunch<2, 8, 4, false>; EXPR_T; }           \
    case 2 * 16 + 2: { using T = TmaLaunch<2, 8, 5, false>; EXPR_T; }           \
    case 2 * 16 + 3: { using T = TmaLaunch<2, 4, 6, false>; EXPR_T; }           \
    case 3 * 16 + 0: { using T = TmaLaunch<3, 4, 4, true>; EXPR_T; }            \
    case 3 * 16 + 1: { using T = TmaLaunch<3, 8, 4, false>; EXPR_T; }           \
    case 4 * 16 + 0: { using T = TmaLaunch<4, 4, 4, true>; EXPR_T; }            \
    case 4 * 16 + 1: { using T = TmaLaunch<4, 8, 4, false>; EXPR_T; }           \
    case 4 * 16 + 2: { using T = TmaLaunch<4, 8, 5, false>; EXPR_T; }           \
    case 4 * 16 + 3: { using T = TmaLaunch<4, 4, 6, false>; EXPR_T; }           \
    case 6 * 16 + 0: { using T = TmaLaunch<6, 4, 4, true>; EXPR_T; }            \
    case 6 * 16 + 1: { using T = TmaLaunch<6, 8, 3, false>; EXPR_T; }           \
    case 8 * 16 + 0: { using T = TmaLaunch<8, 4, 3, true>; EXPR_T; }            \
    case 8 * 16 + 1: { using T = TmaLaunch<8, 8, 3, false>; EXPR_T; }           \
    default: FAIL;                                                              \
  }

bool tma_supported(const phn_params &p) {
  if (p.Nc != 1 || p.precision != PHN_FP32 || p.N % 128 != 0 || p.potential > 1) return false;
  const int K = p.N / 128;
  return K == 1 || K == 2 || K == 3 || K == 4 || K == 6 || K == 8;
}

static bool config_built(int K, int cfg) { return (K == 1 || K == 2 || K == 4) ? cfg < 4 : cfg < 2; }
static bool all_configs(int N) { return N / 128 == 1 || N / 128 == 2 || N / 128 == 4; }

int tma_num_variants(int N) { return all_configs(N) ? kNumTmaVariants : 4; }

// 8-row tiles, pi from HBM, aligned grid (row 4 of kTmaVariants)
int tma_default_variant(int N) { return all_configs(N) ? 4 : 2; }

// Row of kTmaVariants behind a handle-level variant number: sizes with only
// configurations 0 and 1 built expose variants {0, 1, 4, 5}.
static int variant_row(int N, int variant) {
  static const int remap[4] = {0, 1, 4, 5};
  return all_configs(N) ? variant : remap[variant];
}

// Persistent grid for a variant: SMs x resident blocks, or the aligned size
// (0 if the variant cannot run here).
int tma_grid(const phn_params &p, int variant) {
  if (variant < 0 || variant >= tma_num_variants(p.N)) return 0;
  const TmaVariantDef v = kTmaVariants[variant_row(p.N, variant)];
  const int K = p.N / 128;
  if (!config_built(K, v.config)) return 0;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int occ = 0;
  PHN_TMA_SWITCH(K, v.config, occ = T::occupancy(); break, return 0);
  if (occ < 1) return 0;
  const int ty = kTmaConfigs[v.config].ty;
  const long long NT = p.N / ty, W = NT * p.N;
  long long g = (long long)sms * occ;
  if (v.aligned) {
    long long best = 0;
    for (long long m = 1; m <= p.N; ++m)
      if (p.N % m == 0 && NT * m <= g && p.N / m >= 8) best = NT * m;
    if (best == 0) return 0;
    g = best;
  }
  if (g > W) g = W;
  return (int)g;
}

static int tma_config_of(int N, int variant) { return kTmaVariants[variant_row(N, variant)].config; }

cudaError_t launch_step_f32_tma(const Consts &k, int variant, int grid, bool obs, const float *phi, float *phi_out,
                                float *pi, StepF s, double *partials, int *err, cudaStream_t st) {
  const float fk = (float)s.fk, fd = (float)s.fd;
  PHN_TMA_SWITCH(k.N / 128, tma_config_of(k.N, variant),
                 return T::launch(k, obs, grid, phi, phi_out, pi, fk, fd, partials, err, st),
                 return cudaErrorInvalidValue);
}

}  // namespace phn
