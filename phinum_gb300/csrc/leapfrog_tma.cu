// TMA-pipelined leapfrog step for FP32 fields, one component, N a multiple
// of 128 (the production path for the large lattices).
//
// Same arithmetic as step_f32 (leapfrog.cu) -- the two kernels produce
// bit-identical fields -- with a different memory pipeline:
//   * a persistent grid (blocks = SMs x resident blocks); block b owns the
//     contiguous range [W*b/G, W*(b+1)/G) of the plane-tiles
//     w = tile*N + z, tile = 4 full lattice rows, so work is balanced to one
//     plane-tile and each block marches long runs of z;
//   * one producer lane issues 1-D bulk copies (cp.async.bulk, the TMA
//     engine) of each plane-tile into a ring of S shared-memory stages:
//     phi rows y0-1 .. y0+4 (y halo, periodic wrap as two copies) and the
//     tile's pi rows, completing on the stage's "full" mbarrier;
//   * four consumer warps (one per row) read the stage, take x neighbours by
//     warp shuffles (a warp holds whole rows, so the periodic x wrap is a
//     shuffle too), keep phi(z-1), phi(z), phi(z+1) in registers, write
//     pi' and phi' with 16-byte stores, then release the stage on its
//     "empty" mbarrier.
// HBM traffic per site: phi read once (+ the y-halo rows, served by L2),
// pi read once, pi' and phi' written once: the 16-byte algorithmic minimum.
#include "observe.cuh"
#include "phn_internal.h"
#include "tma.cuh"

namespace phn {

constexpr int TMA_TY = 4;                       // lattice rows per tile (= consumer warps)
constexpr int TMA_THREADS = (TMA_TY + 1) * 32;  // + one producer warp

template <int K>
struct TmaShape {
  static constexpr int N = K * 128;
  static constexpr int PHI_ROWS = TMA_TY + 2;
  static constexpr int STAGE_FLOATS = (PHI_ROWS + TMA_TY) * N;
  static constexpr uint32_t PHI_BYTES = PHI_ROWS * N * 4;
  static constexpr uint32_t PI_BYTES = TMA_TY * N * 4;
};

template <int K, int S>
constexpr size_t tma_smem_bytes() {
  return 128 + (size_t)S * TmaShape<K>::STAGE_FLOATS * sizeof(float);
}

__device__ __forceinline__ float get(const float4 &v, int e) {
  return e == 0 ? v.x : (e == 1 ? v.y : (e == 2 ? v.z : v.w));
}

template <int K, int THEORY, bool OBS, int S>
__global__ void __launch_bounds__(TMA_THREADS) step_f32_tma(const float *__restrict__ phi, float *__restrict__ phi_out,
                                                            float *__restrict__ pi, const Consts k, const float fk,
                                                            const float fd, double *__restrict__ partials,
                                                            int *__restrict__ err) {
  using Sh = TmaShape<K>;
  constexpr int N = Sh::N;
  constexpr long long NN = (long long)N * N;
  constexpr long long W = (long long)(N / TMA_TY) * N;
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
      mbar_init(smem_u32(&bars[S + s]), TMA_TY);
    }
    mbar_fence_init();
  }
  __syncthreads();

  AccF accf;
  if (OBS) accf.init();

  if (warp == TMA_TY) {
    // ---------------------------------------------------------- producer
    if (lane == 0) {
      long long L = 0;
      bool ok = true;
      for (long long w = w0; w < w1 && ok;) {
        const int t = (int)(w / N), za = (int)(w % N);
        const long long wend = min(w1, (long long)(t + 1) * N);
        const int zb = za + (int)(wend - w);
        const int y0 = t * TMA_TY;
        for (int j = -1; j <= zb - za && ok; ++j) {
          const int z = (za + j + N) % N;
          const bool center = (j >= 0 && j < zb - za);
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
            bulk_g2s(dst + ROWB, plane, ROWB * (TMA_TY + 1), full);
          } else if (y0 + TMA_TY == N) {
            bulk_g2s(dst, plane + (long long)(y0 - 1) * N, ROWB * (TMA_TY + 1), full);
            bulk_g2s(dst + ROWB * (TMA_TY + 1), plane, ROWB, full);
          } else {
            bulk_g2s(dst, plane + (long long)(y0 - 1) * N, ROWB * (TMA_TY + 2), full);
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
    float4 cm[K], c[K], cp[K];
    const int r = warp;  // row within the tile
    bool ok = true;
    for (long long w = w0; w < w1 && ok;) {
      const int t = (int)(w / N), za = (int)(w % N);
      const long long wend = min(w1, (long long)(t + 1) * N);
      const int zb = za + (int)(wend - w);
      const int y = t * TMA_TY + r;
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
        ok = mbar_wait(smem_u32(&bars[s1]), (uint32_t)((L / S) & 1), err, 2, &abort_flag);
        if (!ok) break;
        const float *nrow = stages + (size_t)s1 * Sh::STAGE_FLOATS + (r + 1) * N;
#pragma unroll
        for (int q = 0; q < K; ++q) cp[q] = *(const float4 *)(nrow + 128 * q + 4 * lane);
        const float *st = stages + (size_t)sz * Sh::STAGE_FLOATS;
        const long long gz = (long long)z * NN + (long long)y * N;
#pragma unroll
        for (int q = 0; q < K; ++q) {
          const int x0 = 128 * q + 4 * lane;
          const float4 ym = *(const float4 *)(st + r * N + x0);
          const float4 yp = *(const float4 *)(st + (r + 2) * N + x0);
          const float4 pv = *(const float4 *)(st + (Sh::PHI_ROWS + r) * N + x0);
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
            if (OBS) {
              const float fxp1[1] = {xp}, fyp1[1] = {ypv}, fzp1[1] = {zp}, c1[1] = {cc}, p1[1] = {pp};
              observe_f32<1, THEORY>(accf, k, c1, p1, fxp1, fyp1, fzp1, gz + NN + x0 + e);
            }
            const float lap = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(xp, xm), __fadd_rn(ypv, ymv)),
                                                            __fadd_rn(zp, zm)),
                                                  __fmul_rn(-6.f, cc)),
                                        k.inv_a2_f);
            const float l = __fmul_rn(cc, cc);
            float coef = fmaf(l, k.c4_f, k.mmM_f);
            if (THEORY == 0) coef = fmaf(__fmul_rn(l, l), k.c6_f, coef);
            float f = fmaf(-coef, cc, lap);
            if (THEORY == 1) f = __fsub_rn(f, k.h_f);
            const float pnv = fmaf(fk, f, pp);
            const float fnv = fmaf(fd, pnv, cc);
            if (e == 0) { pn.x = pnv; fn.x = fnv; }
            if (e == 1) { pn.y = pnv; fn.y = fnv; }
            if (e == 2) { pn.z = pnv; fn.z = fnv; }
            if (e == 3) { pn.w = pnv; fn.w = fnv; }
          }
          *(float4 *)(pi + gz + x0) = pn;
          *(float4 *)(phi_out + gz + x0) = fn;
        }
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
    if (warp < TMA_TY)
      accf.to_double(acc);
    else
      acc.init();
    block_store_n(acc, partials, tid, TMA_THREADS / 32, blockIdx.x);
  }
}

template <int K, int S>
static cudaError_t launch_k(const Consts &k, int theory, bool obs, int grid, const float *phi, float *phi_out,
                            float *pi, float fk, float fd, double *partials, int *err, cudaStream_t st) {
  const size_t smem = tma_smem_bytes<K, S>();
#define PHN_TMA_LAUNCH(TH, OB)                                                                        \
  do {                                                                                                \
    cudaError_t e = cudaFuncSetAttribute(step_f32_tma<K, TH, OB, S>,                                  \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);     \
    if (e != cudaSuccess) return e;                                                                   \
    step_f32_tma<K, TH, OB, S><<<grid, TMA_THREADS, smem, st>>>(phi, phi_out, pi, k, fk, fd, partials, err); \
  } while (0)
  if (theory == 0) {
    if (obs) PHN_TMA_LAUNCH(0, true); else PHN_TMA_LAUNCH(0, false);
  } else {
    if (obs) PHN_TMA_LAUNCH(1, true); else PHN_TMA_LAUNCH(1, false);
  }
#undef PHN_TMA_LAUNCH
  return cudaGetLastError();
}

constexpr int TMA_STAGES = 4;

bool tma_supported(const phn_params &p) {
  return p.Nc == 1 && p.precision == PHN_FP32 && p.N % 128 == 0 && p.N >= 128 && p.N <= 1024 &&
         (p.N / 128 == 1 || p.N / 128 == 2 || p.N / 128 == 3 || p.N / 128 == 4 || p.N / 128 == 6 ||
          p.N / 128 == 8);
}

// Blocks of the persistent grid: SMs x resident blocks per SM.
int tma_grid(const phn_params &p) {
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int K = p.N / 128;
  size_t smem = 0;
  const void *fn = nullptr;
  switch (K) {
    case 1: smem = tma_smem_bytes<1, TMA_STAGES>(); fn = (const void *)step_f32_tma<1, 0, false, TMA_STAGES>; break;
    case 2: smem = tma_smem_bytes<2, TMA_STAGES>(); fn = (const void *)step_f32_tma<2, 0, false, TMA_STAGES>; break;
    case 3: smem = tma_smem_bytes<3, TMA_STAGES>(); fn = (const void *)step_f32_tma<3, 0, false, TMA_STAGES>; break;
    case 4: smem = tma_smem_bytes<4, TMA_STAGES>(); fn = (const void *)step_f32_tma<4, 0, false, TMA_STAGES>; break;
    case 6: smem = tma_smem_bytes<6, TMA_STAGES>(); fn = (const void *)step_f32_tma<6, 0, false, TMA_STAGES>; break;
    default: smem = tma_smem_bytes<8, TMA_STAGES>(); fn = (const void *)step_f32_tma<8, 0, false, TMA_STAGES>; break;
  }
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, TMA_THREADS, smem) != cudaSuccess || occ < 1) occ = 1;
  const long long W = (long long)(p.N / TMA_TY) * p.N;
  long long g = (long long)sms * occ;
  if (g > W) g = W;
  return (int)g;
}

cudaError_t launch_step_f32_tma(const Consts &k, int grid, bool obs, const float *phi, float *phi_out, float *pi,
                                StepF s, double *partials, int *err, cudaStream_t st) {
  const float fk = (float)s.fk, fd = (float)s.fd;
  switch (k.N / 128) {
    case 1: return launch_k<1, TMA_STAGES>(k, k.theory, obs, grid, phi, phi_out, pi, fk, fd, partials, err, st);
    case 2: return launch_k<2, TMA_STAGES>(k, k.theory, obs, grid, phi, phi_out, pi, fk, fd, partials, err, st);
    case 3: return launch_k<3, TMA_STAGES>(k, k.theory, obs, grid, phi, phi_out, pi, fk, fd, partials, err, st);
    case 4: return launch_k<4, TMA_STAGES>(k, k.theory, obs, grid, phi, phi_out, pi, fk, fd, partials, err, st);
    case 6: return launch_k<6, TMA_STAGES>(k, k.theory, obs, grid, phi, phi_out, pi, fk, fd, partials, err, st);
    case 8: return launch_k<8, TMA_STAGES>(k, k.theory, obs, grid, phi, phi_out, pi, fk, fd, partials, err, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace phn
