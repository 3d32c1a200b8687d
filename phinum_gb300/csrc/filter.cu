// Momentum-space filter on the device: apply_filter (filter.cpp:53-133).
//
// Per component of phi and pi: cuFFT R2C of the field, every stored mode
// multiplied by a^3 (fftXtoP_direct's factor) and by the window W(r, |p|),
// C2R back into the field and division by L^3 (fftPtoX_direct).  cuFFT halves
// the x axis where the reference's transposed transform halves y; a mode
// whose y index is above N/2 is held by the reference as its conjugate, so
// its |p| is taken from that conjugate's indices, exactly as the reference's
// loop (filter.cpp:76-99) evaluates it.  On the planes y = 0 and y = N/2 the
// reference stores both p and -p, each with its own window value (their |p|
// can differ in the last bit); the inverse transform then sees the average
// of the two for the real field, so those modes get (W(p) + W(-p)) / 2, which
// is W itself unless a discontinuous window separates them.  Per-axis momenta
// come from the host C library (the reference's values); the windows'
// exp/sin/cos are CUDA's.
#include <cufft.h>
#include <math.h>

#include <vector>

#include "phn_internal.h"

namespace phn {

struct FltArgs {
  int N, which, ntable;
  double r, factor, dp;
};

__device__ __forceinline__ double flt_window(const FltArgs &f, double p, const double *table) {
  if (f.which == PHN_FILTER_TOPHAT) {  // W_tophat, filter.cpp:16-21
    const double r = f.r;
    if (p * r == 0) return 1;
    return 3. * (sin(p * r) / (p * p * p * r * r * r) - cos(p * r) / (p * p * r * r));
  }
  if (f.which == PHN_FILTER_GAUSSIAN) return exp(-p * p * f.r * f.r / 2.);  // W_gaussian, :11-14
  if (f.which == PHN_FILTER_TABLE) {  // W_import_bounce, :46-51
    if (p > (f.ntable - 1) * f.dp) return table[f.ntable - 1];
    return table[(int)(p / f.dp)];
  }
  const double P = 2. * acos(-1.) / f.r;  // W_ktophat, :23-29
  return p < P ? 1 : 0;
}

// |p| of the reference's stored mode (px, py <= N/2, pz): filter.cpp:76-99.
__device__ __forceinline__ double flt_pabs(const double *ptab, int px, int py, int pz) {
  const double ppx = ptab[px], ppy = ptab[py], nu = pz == 0 ? 0.0 : ptab[pz];
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(ppx, ppx), __dmul_rn(ppy, ppy)), __dmul_rn(nu, nu)));
}

// C: float2 or double2 half spectrum [kz][ky][kx <= N/2].
template <typename C>
__global__ void flt_modes(C *__restrict__ F, const double *__restrict__ ptab, const double *__restrict__ table,
                          const FltArgs f) {
  const int N = f.N, M = N / 2 + 1;
  const long long total = (long long)N * N * M;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % M), ky = (int)((i / M) % N), kz = (int)(i / ((long long)M * N));
    double w;
    if (ky == 0 || 2 * ky == N) {  // both p and -p are stored by the reference
      const double w1 = flt_window(f, flt_pabs(ptab, kx, ky, kz), table);
      const double w2 = flt_window(f, flt_pabs(ptab, (N - kx) % N, ky, (N - kz) % N), table);
      w = 0.5 * (w1 + w2);
    } else if (ky > N / 2) {  // the reference holds the conjugate mode
      w = flt_window(f, flt_pabs(ptab, (N - kx) % N, N - ky, (N - kz) % N), table);
    } else {
      w = flt_window(f, flt_pabs(ptab, kx, ky, kz), table);
    }
    C v = F[i];
    v.x = (decltype(v.x))(((double)(decltype(v.x))(f.factor * (double)v.x)) * w);
    v.y = (decltype(v.y))(((double)(decltype(v.y))(f.factor * (double)v.y)) * w);
    F[i] = v;
  }
}

template <typename T>
__global__ void flt_scale(T *__restrict__ x, size_t n, double norm) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    x[i] = (T)((double)x[i] / norm);
}

}  // namespace phn

using namespace phn;

extern "C" int phn_apply_filter(phn_handle *h, double r_filter, int which, const double *table, int ntable,
                                double dp) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (which < PHN_FILTER_TOPHAT || which > PHN_FILTER_KTOPHAT) return set_error(PHN_ERR_INVALID, "filter %d", which);
  if (which == PHN_FILTER_TABLE && (!table || ntable < 1 || !(dp > 0.0)))
    return set_error(PHN_ERR_INVALID, "table filter needs a table and dp > 0");
  const int N = h->p.N, M = N / 2 + 1;
  const bool dbl = h->p.precision == PHN_FP64;
  const size_t nspec = (size_t)N * N * M;
  cudaStream_t st = h->stream;
  void *spec = nullptr;
  double *ptab = nullptr, *d_table = nullptr;
  cufftHandle fwd = 0, inv = 0;
  bool fwd_ok = false, inv_ok = false;
  int r = PHN_OK;
  cudaError_t e = cudaMalloc(&spec, nspec * (dbl ? sizeof(double2) : sizeof(float2)));
  if (e == cudaSuccess) e = cudaMalloc(&ptab, N * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&d_table, (size_t)(which == PHN_FILTER_TABLE ? ntable : 1) * sizeof(double));
  if (e == cudaSuccess) {
    std::vector<double> tab((size_t)N);
    for (int n = 0; n < N; ++n)  // filter.cpp:78-97
      tab[(size_t)n] = n < N / 2 + 1 ? 2.0 / (h->p.a) * sin(n * acos(-1.) / N) : -2.0 / (h->p.a) * sin(n * acos(-1.) / N);
    e = cudaMemcpy(ptab, tab.data(), N * sizeof(double), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess && which == PHN_FILTER_TABLE)
    e = cudaMemcpy(d_table, table, (size_t)ntable * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    r = cuda_error(e, "filter buffers");
  } else if (cufftPlan3d(&fwd, N, N, N, dbl ? CUFFT_D2Z : CUFFT_R2C) != CUFFT_SUCCESS) {
    r = set_error(PHN_ERR_CUDA, "cufftPlan3d (forward) failed");
  } else {
    fwd_ok = true;
    if (cufftPlan3d(&inv, N, N, N, dbl ? CUFFT_Z2D : CUFFT_C2R) != CUFFT_SUCCESS)
      r = set_error(PHN_ERR_CUDA, "cufftPlan3d (inverse) failed");
    else
      inv_ok = true;
  }
  if (r == PHN_OK && (cufftSetStream(fwd, st) != CUFFT_SUCCESS || cufftSetStream(inv, st) != CUFFT_SUCCESS))
    r = set_error(PHN_ERR_CUDA, "cufftSetStream failed");
  FltArgs f;
  f.N = N;
  f.which = which;
  f.ntable = which == PHN_FILTER_TABLE ? ntable : 1;
  f.r = r_filter;
  f.factor = (h->p.a * h->p.a) * h->p.a;                 // fftXtoP_direct's a^3
  f.dp = dp;
  const double norm = (h->p.a * N) * (h->p.a * N) * N * h->p.a;  // fftPtoX_direct's L^3
  const unsigned gb = (unsigned)((nspec + 255) / 256 < 4096 ? (nspec + 255) / 256 : 4096);
  for (int fld = 0; fld < 2 && r == PHN_OK; ++fld)
    for (int a = 0; a < h->p.Nc && r == PHN_OK; ++a) {
      void *x = (char *)(fld == 0 ? h->phi[h->cur] : h->pi) + (size_t)a * h->V * h->elem;
      cufftResult fr = dbl ? cufftExecD2Z(fwd, (double *)x, (cufftDoubleComplex *)spec)
                           : cufftExecR2C(fwd, (float *)x, (cufftComplex *)spec);
      if (fr != CUFFT_SUCCESS) {
        r = set_error(PHN_ERR_CUDA, "cuFFT forward failed (%d)", (int)fr);
        break;
      }
      if (dbl)
        flt_modes<double2><<<gb, 256, 0, st>>>((double2 *)spec, ptab, d_table, f);
      else
        flt_modes<float2><<<gb, 256, 0, st>>>((float2 *)spec, ptab, d_table, f);
      fr = dbl ? cufftExecZ2D(inv, (cufftDoubleComplex *)spec, (double *)x)
               : cufftExecC2R(inv, (cufftComplex *)spec, (float *)x);
      if (fr != CUFFT_SUCCESS) {
        r = set_error(PHN_ERR_CUDA, "cuFFT inverse failed (%d)", (int)fr);
        break;
      }
      if (dbl)
        flt_scale<double><<<1024, 256, 0, st>>>((double *)x, h->V, norm);
      else
        flt_scale<float><<<1024, 256, 0, st>>>((float *)x, h->V, norm);
      e = cudaGetLastError();
      if (e != cudaSuccess) r = cuda_error(e, "filter kernels");
      h->launches += 2;
    }
  // compensated FP32: the filtered values replace the compensated pair
  if (r == PHN_OK && h->p.precision == PHN_FP32_KAHAN) {
    e = cudaMemsetAsync(h->cphi, 0, h->V * h->p.Nc * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->cpi, 0, h->V * h->p.Nc * sizeof(float), st);
    if (e != cudaSuccess) r = cuda_error(e, "filter compensation reset");
  }
  if (r == PHN_OK) {
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) r = cuda_error(e, "filter");
  }
  if (fwd_ok) cufftDestroy(fwd);
  if (inv_ok) cufftDestroy(inv);
  cudaFree(spec);
  cudaFree(ptab);
  cudaFree(d_table);
  return r;
}
