// Self-test of the bounded device waits: a kernel waits on a shared-memory
// mbarrier that nothing ever arrives on -- no copy is issued, no other
// thread takes part -- with a caller-given poll budget.  The wait gives up,
// records its code in the handle's error word exactly as the step kernels'
// waits do, and the kernel returns; the host then reads PHN_ERR_TIMEOUT and
// the context stays usable.  Exercises the failure path without faulting or
// hanging the GPU.
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

}  // namespace phn

using namespace phn;

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
