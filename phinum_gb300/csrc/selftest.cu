// Device self-tests.
//
// Bounded waits: a kernel waits on a shared-memory
// mbarrier that nothing ever arrives on -- no copy is issued, no other
// thread takes part -- with a caller-given poll budget.  The wait gives up,
// records its code in the handle's error word exactly as the step kernels'
// waits do, and the kernel returns; the host then reads PHN_ERR_TIMEOUT and
// the context stays usable.  Exercises the failure path without faulting or
// hanging the GPU.
//
// Division by a constant: div_by (the FP64 kernels' reciprocal multiply with
// residual corrections) against IEEE division over many device-drawn
// operands, including near-midpoint quotients and special values.
#include <math.h>

#include "phn_internal.h"
#include "tma.cuh"

namespace phn {

constexpr int kSelftestCode = 99;

__global__ void wait_selftest(int *err, long long polls) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  const uint32_t b = smem_u32(&bar);
  mbar_init(b, 1);
  mbar_fence_init();
  // phase 0 never completes: the single expected arrival never happens
  mbar_wait(b, 0, err, kSelftestCode, nullptr, polls);
}

// Operand i of the division self-test: a splitmix64 hash of (seed, i).
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ double divide_operand(double b, unsigned long long seed, long long i) {
  const unsigned long long h = mix64(seed ^ mix64((unsigned long long)i));
  const unsigned long long h2 = mix64(h);
  const int kind = (int)(h2 & 15);
  const unsigned long long sign = (h2 >> 4) & 1;
  const unsigned long long mant = h & ((1ull << 52) - 1);
  if (kind == 0) {  // specials: zeros, subnormals, infinities, NaN
    const double sp[6] = {0.0, 4.9e-324, 2.2e-310, __longlong_as_double(0x7ff0000000000000ll),
                          __longlong_as_double(0x7ff8000000000000ll), 1e-305};
    const double v = sp[(h2 >> 8) % 6];
    return sign ? -v : v;
  }
  const int e = (int)((h2 >> 8) % 2001) - 1000;  // exponent in [-1000, 1000]
  const double m = __longlong_as_double((long long)((1023ull << 52) | mant));  // [1, 2)
  const double r = ldexp(m, e);
  if (kind < 8) return sign ? -r : r;
  // near a midpoint: b * (q + ulp(q)/2), moved by -2..2 ulps
  const double q = ldexp(m, e / 2);
  const double up = __longlong_as_double(__double_as_longlong(q) + 1) - q;
  double a = b * (q + 0.5 * up);
  const int k = (int)((h2 >> 20) % 5) - 2;
  a = __longlong_as_double(__double_as_longlong(a) + k);
  return sign ? -a : a;
}

__global__ void divide_selftest(const Consts k, double b, double rb, double rl, bool near, long long n,
                                unsigned long long seed, unsigned long long *bad) {
  unsigned long long local = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double a = divide_operand(b, seed, i);
    const double fast = near ? div_by_near(k, a, b, rb) : div_by(k, a, b, rb, rl), ieee = a / b;
    const bool same = __double_as_longlong(fast) == __double_as_longlong(ieee) || (fast != fast && ieee != ieee);
    local += same ? 0 : 1;
  }
  if (local) atomicAdd(bad, local);
}

}  // namespace phn

using namespace phn;

extern "C" int phn_divide_selftest(phn_handle *h, double b, long long n, unsigned long long seed,
                                   long long *mismatches) {
  if (!h || !mismatches || n < 1 || n > (1ll << 34) || !(b != 0.0) || !isfinite(b))
    return set_error(PHN_ERR_INVALID, "bad argument");
  Consts k = h->k;
  const double m = fabs(b);
  k.fastdiv = (m >= 0x1p-100 && m <= 0x1p100) ? 1 : 0;
  // div_by_near where the reciprocal is within 2^-54, as the kernels use it
  // for such divisors; div_by with the two-word reciprocal otherwise
  const bool near = fabs(fma(b, 1.0 / b, -1.0)) <= 0x1p-54;
  const double rb = 1.0 / b, rl = fma(-b, rb, 1.0) / b;
  unsigned long long *d_bad = nullptr;
  cudaError_t e = cudaMalloc((void **)&d_bad, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(unsigned long long), h->stream);
  if (e == cudaSuccess) {
    divide_selftest<<<152 * 8, 256, 0, h->stream>>>(k, b, rb, rl, near, n, seed, d_bad);
    e = cudaGetLastError();
  }
  unsigned long long bad = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d_bad);
  if (e != cudaSuccess) return cuda_error(e, "divide self-test");
  h->launches++;
  *mismatches = (long long)bad;
  return PHN_OK;
}

extern "C" int phn_wait_selftest(phn_handle *h, long long polls) {
  if (!h || polls < 1 || polls > kWaitPolls) return set_error(PHN_ERR_INVALID, "polls outside [1, %lld]", kWaitPolls);
  wait_selftest<<<1, 32, 0, h->stream>>>(h->d_err, polls);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_error(e, "wait self-test");
  h->launches++;
  int word = 0;
  e = cudaMemcpy(&word, h->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "error word");
  e = cudaMemset(h->d_err, 0, sizeof(int));
  if (e != cudaSuccess) return cuda_error(e, "error word reset");
  if (word == kSelftestCode) return set_error(PHN_ERR_TIMEOUT, "a bounded device wait gave up (code %d)", word);
  return set_error(PHN_ERR_CUDA, "wait self-test: error word %d", word);
}
