// Radial power spectrum: cuFFT R2C of each component of phi and pi, then a
// binning kernel that reproduces Calculate_CorrelationFunctions
// (momentumspace.cpp:140-278) mode for mode.
//
// The reference transforms a transposed copy so that lattice y is FFTW's
// halved axis (clusterfft.cpp:198) and visits (px in [0,N), py in [0,N/2],
// pz in [0,N)), counting a mode twice unless py is 0 or N/2.  cuFFT halves the
// fastest axis, lattice x, instead.  The binning kernel walks the
// reference's own mode set: a mode with px <= N/2 is read directly, a mode
// with px > N/2 from its conjugate partner (N-px, -py, -pz), which has the
// same |F|^2 and Re(Phi Pi*).  Bin indices are evaluated in FP64 exactly as
// the reference does, from the same per-axis lattice momenta, so bin counts
// and bin membership are identical; the sums differ from FFTW's only by
// rounding.
//
// A second bin rule serves the configuration's radial spectrum (no reference
// counterpart): the same modes, weights and sums, binned uniformly in |p| on
// [0, p_max] with p_max the largest lattice momentum.
//
// Accumulation is deterministic: per-warp shared-memory histograms (one lane
// per distinct bin adds a fixed-shape butterfly sum of the warp's values),
// folded per block in warp order, then over blocks in block order.
#include <cufft.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "phn_internal.h"

namespace phn {

constexpr int SPEC_THREADS = 256;
constexpr int SPEC_WARPS = SPEC_THREADS / 32;

struct SpecState {
  cufftHandle plan;
  bool plan_ok;
  void *fphi, *fpi;        // complex half-spectra, [z][y][x/2+1]
  double *ptab;            // lattice momentum per axis index (device)
  double *partials;        // [blocks][3][nbins]
  double *bins;            // [3][nbins] final, per component
  int *counts;             // [nbins] (device)
  int *flag;               // bin overflow flag (device)
  int nblocks, nbins;
  double binsize;
  std::vector<int> h_counts;
  bool counts_ok;
  // uniform-bin (configuration) mode, allocated on first use
  int u_nbins;
  double *u_partials, *u_bins;
  int *u_counts;
};

constexpr int SPEC_MAX_UNIFORM_BINS = 1024;  // per-warp histograms in shared memory
enum { RULE_REFERENCE = 0, RULE_UNIFORM = 1 };

// Lattice momentum of index n along an axis (momentumspace.cpp:222-244).
static double lattice_p(int n, int N, double a) {
  if (n < N / 2 + 1) return 2.0 / (a) * sin(n * acos(-1.) / N);
  return -2.0 / (a) * sin(n * acos(-1.) / N);
}

__device__ __forceinline__ double mag2(float2 v) { return (double)v.x * v.x + (double)v.y * v.y; }
__device__ __forceinline__ double mag2(double2 v) { return v.x * v.x + v.y * v.y; }
__device__ __forceinline__ double dotre(float2 a, float2 b) { return (double)a.x * b.x + (double)a.y * b.y; }
__device__ __forceinline__ double dotre(double2 a, double2 b) { return a.x * b.x + a.y * b.y; }

// COUNT: only the mode counts (InitBCounts), no field reads.
// rule RULE_REFERENCE: bin = int(|p| / binsize + 0.5) (momentumspace.cpp:228);
// rule RULE_UNIFORM: bin = int(|p| / binsize), binsize = p_max / nbins, the
// top edge folded into the last bin.
template <typename C, bool COUNT>
__global__ void __launch_bounds__(SPEC_THREADS) bin_kernel(const C *__restrict__ fphi, const C *__restrict__ fpi,
                                                          const double *__restrict__ ptab, int N, double binsize,
                                                          int nbins, int rule, double scale,
                                                          double *__restrict__ partials, int *__restrict__ counts,
                                                          int *__restrict__ flag) {
  extern __shared__ double hist[];  // [SPEC_WARPS][3][nbins]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < SPEC_WARPS * 3 * nbins; i += SPEC_THREADS) hist[i] = 0.0;
  __syncthreads();
  double *hF = hist + (size_t)warp * 3 * nbins, *hK = hF + nbins, *hQ = hK + nbins;
  const int h = N / 2, M = N / 2 + 1;
  const long long total = (long long)N * M * N;
  const long long stride = (long long)gridDim.x * SPEC_THREADS;
  // uniform trip count across the warp so that warp collectives stay converged
  const long long iters = (total + stride - 1) / stride;
  for (long long it = 0; it < iters; ++it) {
    const long long i = it * stride + (long long)blockIdx.x * SPEC_THREADS + threadIdx.x;
    int key = -1;
    double f = 0.0, k = 0.0, q = 0.0;
    if (i < total) {
      const int px = (int)(i % N);
      const long long t = i / N;
      const int py = (int)(t % M);
      const int pz = (int)(t / M);
      const double ppx = ptab[px], ppy = ptab[py], nu = ptab[pz];
      const double psqr = __dadd_rn(__dadd_rn(__dmul_rn(ppx, ppx), __dmul_rn(ppy, ppy)), __dmul_rn(nu, nu));
      int bin;
      if (rule == RULE_REFERENCE) {
        bin = (int)(__dadd_rn(sqrt(psqr) / binsize, 0.5));
      } else {
        bin = (int)(sqrt(psqr) / binsize);
        if (bin >= nbins) bin = nbins - 1;
      }
      const int w = (py != 0 && py != h) ? 2 : 1;
      if (bin >= nbins) {
        atomicOr(flag, 1);
      } else if (COUNT) {
        atomicAdd(&counts[bin], w);
      } else {
        long long m;
        if (px <= h)
          m = ((long long)pz * N + py) * M + px;
        else
          m = ((long long)((N - pz) % N) * N + (N - py) % N) * M + (N - px);
        const C a = fphi[m], b = fpi[m];
        key = bin;
        f = w * mag2(a) * scale;
        k = w * mag2(b) * scale;
        q = w * dotre(a, b) * scale;
      }
    }
    if (COUNT) continue;
    unsigned todo = __ballot_sync(0xffffffffu, key >= 0);
    while (todo) {
      const int src = __ffs(todo) - 1;
      const int b = __shfl_sync(0xffffffffu, key, src);
      const bool mine = (key == b);
      const unsigned grp = __ballot_sync(0xffffffffu, mine);
      double vf = mine ? f : 0.0, vk = mine ? k : 0.0, vq = mine ? q : 0.0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        vf += __shfl_xor_sync(0xffffffffu, vf, off);
        vk += __shfl_xor_sync(0xffffffffu, vk, off);
        vq += __shfl_xor_sync(0xffffffffu, vq, off);
      }
      if (lane == src) {
        hF[b] += vf;
        hK[b] += vk;
        hQ[b] += vq;
      }
      todo &= ~grp;
      __syncwarp();
    }
  }
  if (COUNT) return;
  __syncthreads();
  // fold the warp histograms in warp order; one record per block
  for (int j = threadIdx.x; j < 3 * nbins; j += SPEC_THREADS) {
    double s = 0.0;
    for (int w = 0; w < SPEC_WARPS; ++w) s += hist[(size_t)w * 3 * nbins + j];
    partials[(size_t)blockIdx.x * 3 * nbins + j] = s;
  }
}

__global__ void fold_blocks(const double *__restrict__ partials, int nblocks, int nbins, double *__restrict__ out) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < 3 * nbins; j += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += partials[(size_t)b * 3 * nbins + j];
    out[j] = s;
  }
}

void spectrum_release(phn_handle *h) {
  SpecState *s = (SpecState *)h->spec;
  if (!s) return;
  if (s->plan_ok) cufftDestroy(s->plan);
  cudaFree(s->fphi);
  cudaFree(s->fpi);
  cudaFree(s->ptab);
  cudaFree(s->partials);
  cudaFree(s->bins);
  cudaFree(s->counts);
  cudaFree(s->flag);
  cudaFree(s->u_partials);
  cudaFree(s->u_bins);
  cudaFree(s->u_counts);
  delete s;
  h->spec = nullptr;
}

// MomentumSpace::init (momentumspace.cpp:40-47).
static void bin_geometry(const phn_params &p, int *nbins, double *binsize) {
  const double pTmin = (2.0 / (p.a)) * sin(acos(-1.) / p.N);
  const double pTmax = sqrt(3.0 * (4.0 / (p.a * p.a)));
  *binsize = pTmin;
  *nbins = (int)(pTmax / pTmin + 0.5) + 2;
}

static int spec_init(phn_handle *h) {
  if (h->spec) return PHN_OK;
  SpecState *s = new SpecState();
  h->spec = s;
  const int N = h->p.N;
  bin_geometry(h->p, &s->nbins, &s->binsize);
  s->nblocks = 152 * 4;
  const size_t ncomplex = (size_t)N * N * (N / 2 + 1);
  const bool dbl = h->p.precision == PHN_FP64;
  const size_t csize = dbl ? sizeof(double2) : sizeof(float2);
  cudaError_t e;
#define CKS(call)                                      \
  do {                                                 \
    e = (call);                                        \
    if (e != cudaSuccess) return cuda_error(e, #call); \
  } while (0)
  CKS(cudaMalloc(&s->fphi, ncomplex * csize));
  CKS(cudaMalloc(&s->fpi, ncomplex * csize));
  CKS(cudaMalloc(&s->ptab, N * sizeof(double)));
  CKS(cudaMalloc(&s->partials, (size_t)s->nblocks * 3 * s->nbins * sizeof(double)));
  CKS(cudaMalloc(&s->bins, (size_t)3 * s->nbins * sizeof(double)));
  CKS(cudaMalloc(&s->counts, (size_t)s->nbins * sizeof(int)));
  CKS(cudaMalloc(&s->flag, sizeof(int)));
  std::vector<double> tab(N);
  for (int n = 0; n < N; ++n) tab[n] = lattice_p(n, N, h->p.a);
  CKS(cudaMemcpy(s->ptab, tab.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  if (cufftPlan3d(&s->plan, N, N, N, dbl ? CUFFT_D2Z : CUFFT_R2C) != CUFFT_SUCCESS)
    return set_error(PHN_ERR_CUDA, "cufftPlan3d(%d^3) failed", N);
  s->plan_ok = true;
  if (cufftSetStream(s->plan, h->stream) != CUFFT_SUCCESS) return set_error(PHN_ERR_CUDA, "cufftSetStream failed");
  const size_t smem = (size_t)SPEC_WARPS * 3 * s->nbins * sizeof(double);
  // the largest histogram either rule uses
  const size_t smem_max = (size_t)SPEC_WARPS * 3 * (s->nbins > SPEC_MAX_UNIFORM_BINS ? s->nbins : SPEC_MAX_UNIFORM_BINS) *
                          sizeof(double);
  CKS(cudaFuncSetAttribute(bin_kernel<float2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
  CKS(cudaFuncSetAttribute(bin_kernel<double2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
  CKS(cudaFuncSetAttribute(bin_kernel<float2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
  // mode counts (InitBCounts, momentumspace.cpp:89-138): field independent
  CKS(cudaMemsetAsync(s->counts, 0, s->nbins * sizeof(int), h->stream));
  CKS(cudaMemsetAsync(s->flag, 0, sizeof(int), h->stream));
  bin_kernel<float2, true><<<s->nblocks, SPEC_THREADS, smem, h->stream>>>(
      nullptr, nullptr, s->ptab, N, s->binsize, s->nbins, RULE_REFERENCE, 0.0, nullptr, s->counts, s->flag);
  CKS(cudaGetLastError());
  h->launches++;
  s->h_counts.resize(s->nbins);
  int flag = 0;
  CKS(cudaMemcpyAsync(s->h_counts.data(), s->counts, s->nbins * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CKS(cudaMemcpyAsync(&flag, s->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CKS(cudaStreamSynchronize(h->stream));
  if (flag) return set_error(PHN_ERR_INVALID, "bin array too small (momentumspace.cpp:128)");
#undef CKS
  return PHN_OK;
}

}  // namespace phn

using namespace phn;

extern "C" {

int phn_spectrum_bins(const phn_handle *h, int *nbins, double *binsize) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  int nb;
  double bs;
  bin_geometry(h->p, &nb, &bs);
  if (nbins) *nbins = nb;
  if (binsize) *binsize = bs;
  return PHN_OK;
}

int phn_spectrum(phn_handle *h, double *F, double *K, double *Q, int *counts, int nbins) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  int r = spec_init(h);
  if (r) {
    spectrum_release(h);
    return r;
  }
  SpecState *s = (SpecState *)h->spec;
  if (nbins < s->nbins) return set_error(PHN_ERR_TRUNCATED, "nbins=%d < %d", nbins, s->nbins);
  const int N = h->p.N, Nc = h->p.Nc;
  const bool dbl = h->p.precision == PHN_FP64;
  const double f3 = (h->p.a * h->p.a) * h->p.a;  // fftXtoP_direct's a^3 (clusterfft.cpp:187,222)
  const double scale = f3 * f3;
  const size_t smem = (size_t)SPEC_WARPS * 3 * s->nbins * sizeof(double);
  std::vector<double> hb((size_t)3 * s->nbins);
  for (int k = 0; k < s->nbins * Nc; ++k) {
    if (F) F[k] = 0.0;
    if (K) K[k] = 0.0;
    if (Q) Q[k] = 0.0;
  }
  for (int a = 0; a < Nc; ++a) {
    cufftResult fr;
    if (dbl) {
      double *phi = (double *)h->phi[h->cur] + (size_t)a * h->V, *pi = (double *)h->pi + (size_t)a * h->V;
      fr = cufftExecD2Z(s->plan, phi, (cufftDoubleComplex *)s->fphi);
      if (fr == CUFFT_SUCCESS) fr = cufftExecD2Z(s->plan, pi, (cufftDoubleComplex *)s->fpi);
    } else {
      float *phi = (float *)h->phi[h->cur] + (size_t)a * h->V, *pi = (float *)h->pi + (size_t)a * h->V;
      fr = cufftExecR2C(s->plan, phi, (cufftComplex *)s->fphi);
      if (fr == CUFFT_SUCCESS) fr = cufftExecR2C(s->plan, pi, (cufftComplex *)s->fpi);
    }
    if (fr != CUFFT_SUCCESS) return set_error(PHN_ERR_CUDA, "cuFFT exec failed (%d)", (int)fr);
    if (dbl)
      bin_kernel<double2, false><<<s->nblocks, SPEC_THREADS, smem, h->stream>>>(
          (const double2 *)s->fphi, (const double2 *)s->fpi, s->ptab, N, s->binsize, s->nbins, RULE_REFERENCE, scale,
          s->partials, nullptr, s->flag);
    else
      bin_kernel<float2, false><<<s->nblocks, SPEC_THREADS, smem, h->stream>>>(
          (const float2 *)s->fphi, (const float2 *)s->fpi, s->ptab, N, s->binsize, s->nbins, RULE_REFERENCE, scale,
          s->partials, nullptr, s->flag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "bin_kernel");
    fold_blocks<<<(3 * s->nbins + 255) / 256, 256, 0, h->stream>>>(s->partials, s->nblocks, s->nbins, s->bins);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "fold_blocks");
    h->launches += 2;
    e = cudaMemcpyAsync(hb.data(), s->bins, hb.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_error(e, "spectrum readback");
    for (int b = 0; b < s->nbins; ++b) {
      if (F) F[b * Nc + a] = hb[b];
      if (K) K[b * Nc + a] = hb[s->nbins + b];
      if (Q) Q[b * Nc + a] = hb[2 * s->nbins + b];
    }
  }
  if (counts)
    for (int b = 0; b < s->nbins; ++b) counts[b] = s->h_counts[b];
  return PHN_OK;
}

int phn_spectrum_uniform(phn_handle *h, int nbins, double *F, double *K, double *Q, int *counts) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (nbins < 1 || nbins > SPEC_MAX_UNIFORM_BINS)
    return set_error(PHN_ERR_INVALID, "nbins=%d outside [1, %d]", nbins, SPEC_MAX_UNIFORM_BINS);
  int r = spec_init(h);
  if (r) {
    spectrum_release(h);
    return r;
  }
  SpecState *s = (SpecState *)h->spec;
  const int N = h->p.N, Nc = h->p.Nc;
  const bool dbl = h->p.precision == PHN_FP64;
  cudaError_t e;
  if (s->u_nbins != nbins) {
    cudaFree(s->u_partials);
    cudaFree(s->u_bins);
    cudaFree(s->u_counts);
    s->u_partials = s->u_bins = nullptr;
    s->u_counts = nullptr;
    s->u_nbins = 0;
    e = cudaMalloc(&s->u_partials, (size_t)s->nblocks * 3 * nbins * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->u_bins, (size_t)3 * nbins * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->u_counts, (size_t)nbins * sizeof(int));
    if (e != cudaSuccess) return cuda_error(e, "uniform spectrum buffers");
    s->u_nbins = nbins;
  }
  // p_max = pTmax of momentumspace.cpp:43, the largest lattice |p|
  const double pmax = sqrt(3.0 * (4.0 / (h->p.a * h->p.a)));
  const double width = pmax / nbins;
  const double f3 = (h->p.a * h->p.a) * h->p.a;
  const double scale = f3 * f3;
  const size_t smem = (size_t)SPEC_WARPS * 3 * nbins * sizeof(double);
  std::vector<int> hc(nbins);
  e = cudaMemsetAsync(s->u_counts, 0, nbins * sizeof(int), h->stream);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemsetAsync");
  bin_kernel<float2, true><<<s->nblocks, SPEC_THREADS, smem, h->stream>>>(
      nullptr, nullptr, s->ptab, N, width, nbins, RULE_UNIFORM, 0.0, nullptr, s->u_counts, s->flag);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "bin_kernel (counts)");
  h->launches++;
  e = cudaMemcpyAsync(hc.data(), s->u_counts, nbins * sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  if (e != cudaSuccess) return cuda_error(e, "counts readback");
  std::vector<double> hb((size_t)3 * nbins);
  for (int a = 0; a < Nc; ++a) {
    cufftResult fr;
    if (dbl) {
      double *phi = (double *)h->phi[h->cur] + (size_t)a * h->V, *pi = (double *)h->pi + (size_t)a * h->V;
      fr = cufftExecD2Z(s->plan, phi, (cufftDoubleComplex *)s->fphi);
      if (fr == CUFFT_SUCCESS) fr = cufftExecD2Z(s->plan, pi, (cufftDoubleComplex *)s->fpi);
    } else {
      float *phi = (float *)h->phi[h->cur] + (size_t)a * h->V, *pi = (float *)h->pi + (size_t)a * h->V;
      fr = cufftExecR2C(s->plan, phi, (cufftComplex *)s->fphi);
      if (fr == CUFFT_SUCCESS) fr = cufftExecR2C(s->plan, pi, (cufftComplex *)s->fpi);
    }
    if (fr != CUFFT_SUCCESS) return set_error(PHN_ERR_CUDA, "cuFFT exec failed (%d)", (int)fr);
    if (dbl)
      bin_kernel<double2, false><<<s->nblocks, SPEC_THREADS, smem, h->stream>>>(
          (const double2 *)s->fphi, (const double2 *)s->fpi, s->ptab, N, width, nbins, RULE_UNIFORM, scale,
          s->u_partials, nullptr, s->flag);
    else
      bin_kernel<float2, false><<<s->nblocks, SPEC_THREADS, smem, h->stream>>>(
          (const float2 *)s->fphi, (const float2 *)s->fpi, s->ptab, N, width, nbins, RULE_UNIFORM, scale,
          s->u_partials, nullptr, s->flag);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "bin_kernel");
    fold_blocks<<<(3 * nbins + 255) / 256, 256, 0, h->stream>>>(s->u_partials, s->nblocks, nbins, s->u_bins);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "fold_blocks");
    h->launches += 2;
    e = cudaMemcpyAsync(hb.data(), s->u_bins, hb.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_error(e, "spectrum readback");
    for (int b = 0; b < nbins; ++b) {
      if (F) F[b * Nc + a] = hb[b];
      if (K) K[b * Nc + a] = hb[nbins + b];
      if (Q) Q[b * Nc + a] = hb[2 * nbins + b];
    }
  }
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_error(e, "spectrum readback");
  if (counts)
    for (int b = 0; b < nbins; ++b) counts[b] = hc[b];
  return PHN_OK;
}

}  // extern "C"
