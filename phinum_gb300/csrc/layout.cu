// Conversion between the reference layout (Nc*N*N*(N+2) pseudo_double values,
// component innermost, ghost z-slabs; lattice.cpp:76-78, util.cpp:34-37) --
// doubles from the reference's double-precision build, floats from its
// single-precision one (parameters.cpp:13-33) -- and the device layout: one
// contiguous [z][y][x] plane stack per component, no ghosts, in the handle's
// precision.  Runs on the device after (before) a single H2D (D2H) copy of
// the reference-layout array.
#include "phn_internal.h"

namespace phn {

template <typename R, typename T>
__global__ void from_ref_kernel(const R *__restrict__ ref, T *__restrict__ dst, int N, int Nc) {
  const size_t NN = (size_t)N * N, V = NN * N;
  const size_t total = V * (size_t)Nc;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t site = i / Nc;            // interior site, [z][y][x]
    const int a = (int)(i - site * Nc);
    dst[a * V + site] = (T)ref[i + (size_t)Nc * NN];  // skip ghost slab 0
  }
}

// Compensated FP32: hi = fl(v), comp = fl(hi - v), so that hi - comp keeps
// the FP64 input to about 2^-48 relative.
template <typename R>
__global__ void from_ref_kahan_kernel(const R *__restrict__ ref, float *__restrict__ hi, float *__restrict__ comp,
                                      int N, int Nc) {
  const size_t NN = (size_t)N * N, V = NN * N;
  const size_t total = V * (size_t)Nc;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t site = i / Nc;
    const int a = (int)(i - site * Nc);
    const double v = (double)ref[i + (size_t)Nc * NN];
    const float h = (float)v;
    hi[a * V + site] = h;
    comp[a * V + site] = (float)((double)h - v);
  }
}

template <typename T, typename R>
__global__ void to_ref_kernel(const T *__restrict__ src, const float *__restrict__ comp, R *__restrict__ ref,
                              int N, int Nc) {
  const size_t NN = (size_t)N * N, V = NN * N;
  const size_t total = (size_t)Nc * NN * (N + 2);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t r = i / Nc;
    const int a = (int)(i - r * Nc);
    const size_t zr = r / NN;              // 0..N+1 in the reference layout
    const size_t inplane = r - zr * NN;
    const size_t z = (zr == 0) ? (size_t)N - 1 : (zr == (size_t)N + 1 ? 0 : zr - 1);  // exchange()
    const size_t s = a * V + z * NN + inplane;
    double v = (double)src[s];
    if (comp) v -= (double)comp[s];
    ref[i] = (R)v;
  }
}

static int blocks_for(size_t n) {
  size_t b = (n + 255) / 256;
  if (b > 152 * 64) b = 152 * 64;
  return (int)(b ? b : 1);
}

template <typename R>
cudaError_t launch_from_ref(const R *ref, void *dst, int prec, int N, int Nc, cudaStream_t st) {
  const size_t n = (size_t)N * N * N * Nc;
  if (prec == PHN_FP64)
    from_ref_kernel<R, double><<<blocks_for(n), 256, 0, st>>>(ref, (double *)dst, N, Nc);
  else
    from_ref_kernel<R, float><<<blocks_for(n), 256, 0, st>>>(ref, (float *)dst, N, Nc);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_from_ref_kahan(const R *ref, float *hi, float *comp, int N, int Nc, cudaStream_t st) {
  const size_t n = (size_t)N * N * N * Nc;
  from_ref_kahan_kernel<R><<<blocks_for(n), 256, 0, st>>>(ref, hi, comp, N, Nc);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_to_ref(const void *src, R *ref, int prec, int N, int Nc, cudaStream_t st) {
  const size_t n = (size_t)Nc * N * N * (N + 2);
  if (prec == PHN_FP64)
    to_ref_kernel<double, R><<<blocks_for(n), 256, 0, st>>>((const double *)src, nullptr, ref, N, Nc);
  else
    to_ref_kernel<float, R><<<blocks_for(n), 256, 0, st>>>((const float *)src, nullptr, ref, N, Nc);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_to_ref_kahan(const float *hi, const float *comp, R *ref, int N, int Nc, cudaStream_t st) {
  const size_t n = (size_t)Nc * N * N * (N + 2);
  to_ref_kernel<float, R><<<blocks_for(n), 256, 0, st>>>(hi, comp, ref, N, Nc);
  return cudaGetLastError();
}

template cudaError_t launch_from_ref<double>(const double *, void *, int, int, int, cudaStream_t);
template cudaError_t launch_from_ref<float>(const float *, void *, int, int, int, cudaStream_t);
template cudaError_t launch_from_ref_kahan<double>(const double *, float *, float *, int, int, cudaStream_t);
template cudaError_t launch_from_ref_kahan<float>(const float *, float *, float *, int, int, cudaStream_t);
template cudaError_t launch_to_ref<double>(const void *, double *, int, int, int, cudaStream_t);
template cudaError_t launch_to_ref<float>(const void *, float *, int, int, int, cudaStream_t);
template cudaError_t launch_to_ref_kahan<double>(const float *, const float *, double *, int, int, cudaStream_t);
template cudaError_t launch_to_ref_kahan<float>(const float *, const float *, float *, int, int, cudaStream_t);

}  // namespace phn
