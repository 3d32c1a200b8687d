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
// steps always use a persistent variant (few block records to fold) and
// per-plane FP32 partials with one compensated update per plane.
#include "kick.cuh"
#include "observe.cuh"
#include "phn_internal.h"

namespace phn {

struct X4Variant {
  int w, cz;
  bool persistent;
};
constexpr X4Variant kX4Variants[] = {{8, 32, true}, {8, 16, true}, {4, 32, true},
                                     {8, 16, false}, {8, 8, false}, {4, 16, false}};
constexpr int kNumX4Variants = 6;

template <int W, int MODE, int THEORY>
__global__ void __launch_bounds__(32 * W) step_f32_x4(const Consts k, const float *__restrict__ phi,
                                                      float *__restrict__ phi_out, float *__restrict__ pi, StepF s,
                                                      int cz, int nitems, double *__restrict__ partials) {
  const float fk = MODE == MODE_OBS ? 0.f : (float)s.fk;
  const float fd = MODE == MODE_OBS ? 0.f : (float)s.fd;
  const int N = k.N, NN = N * N;
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const int chunks = NN / (128 * W);
  AccF accf;
  if (MODE != MODE_STEP) accf.init();
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
      if (MODE != MODE_STEP) {
        const long long kidx = (long long)q + (long long)(z + 1) * NN;
        PlaneF P;
        P.clear();
        observe_site<THEORY>(P, accf, k, c.x, p.x, c.y, yp.x, cp.x, kidx);
        observe_site<THEORY>(P, accf, k, c.y, p.y, c.z, yp.y, cp.y, kidx + 1);
        observe_site<THEORY>(P, accf, k, c.z, p.z, c.w, yp.z, cp.z, kidx + 2);
        observe_site<THEORY>(P, accf, k, c.w, p.w, xp, yp.w, cp.w, kidx + 3);
        flush_plane(accf, P);
      }
      if (MODE != MODE_OBS) {
        float4 pn, fn;
        kick_drift_f32<THEORY>(k, fk, fd, c.x, xm, c.y, ym.x, yp.x, cm.x, cp.x, p.x, pn.x, fn.x);
        kick_drift_f32<THEORY>(k, fk, fd, c.y, c.x, c.z, ym.y, yp.y, cm.y, cp.y, p.y, pn.y, fn.y);
        kick_drift_f32<THEORY>(k, fk, fd, c.z, c.y, c.w, ym.z, yp.z, cm.z, cp.z, p.z, pn.z, fn.z);
        kick_drift_f32<THEORY>(k, fk, fd, c.w, c.z, xp, ym.w, yp.w, cm.w, cp.w, p.w, pn.w, fn.w);
        *(float4 *)(pi + i) = pn;
        *(float4 *)(phi_out + i) = fn;
      }
      cm = c;
      c = cp;
    }
  }
  if (MODE != MODE_STEP) {
    // one record per block, whatever the number of items it walked
    Acc acc;
    accf.to_double(acc);
    block_store_n(acc, partials, tid, W, (size_t)blockIdx.x);
  }
}

bool x4_supported(const phn_params &p) {
  return p.precision == PHN_FP32 && p.Nc == 1 && p.N % 32 == 0 && p.N >= 32 && (p.potential == 0 || p.potential == 1);
}

int x4_num_variants() { return kNumX4Variants; }

int x4_obs_variant(int variant) {
  if (kX4Variants[variant].persistent) return variant;
  for (int v = 0; v < kNumX4Variants; ++v)
    if (kX4Variants[v].persistent && kX4Variants[v].w == kX4Variants[variant].w) return v;
  return 0;
}

static int x4_items(int N, const X4Variant &v) {
  const int cz = v.cz < N ? v.cz : N;
  return ((N + cz - 1) / cz) * (N * N / (128 * v.w));
}

template <int W>
static const void *x4_fn() {
  return (const void *)step_f32_x4<W, MODE_STEP, 0>;
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
  const void *fn = v.w == 8 ? x4_fn<8>() : x4_fn<4>();
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 32 * v.w, 0) != cudaSuccess || occ < 1) occ = 1;
  const int g = sms * occ;
  return g < items ? g : items;
}

template <int W, int MODE>
static cudaError_t x4_launch_t(const Consts &k, int theory, int grid, int cz, int nitems, const float *phi,
                               float *phi_out, float *pi, StepF s, double *partials, cudaStream_t st) {
  if (theory == 0)
    step_f32_x4<W, MODE, 0><<<grid, dim3(32, W), 0, st>>>(k, phi, phi_out, pi, s, cz, nitems, partials);
  else
    step_f32_x4<W, MODE, 1><<<grid, dim3(32, W), 0, st>>>(k, phi, phi_out, pi, s, cz, nitems, partials);
  return cudaGetLastError();
}

cudaError_t launch_step_f32_x4(const Consts &k, int variant, int grid, int mode, const float *phi, float *phi_out,
                               float *pi, StepF s, double *partials, cudaStream_t st) {
  const X4Variant &v = kX4Variants[variant];
  const int cz = v.cz < k.N ? v.cz : k.N;
  const int nitems = x4_items(k.N, v);
#define PHN_X4(WV, MD) return x4_launch_t<WV, MD>(k, k.theory, grid, cz, nitems, phi, phi_out, pi, s, partials, st)
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
