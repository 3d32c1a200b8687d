// Volume averages over caller-owned device fields without any allocation.
//
// phn_volume_averages needs a handle, and a handle allocates its fields and
// its scratch with cudaMalloc.  Some hosts cannot do that at the point where
// they want the averages: a host whose framework owns every byte of device
// memory through its own pool (it hands out field buffers but forbids other
// allocators on the device), or a host inside a stream-ordered time loop
// where a cudaMalloc/cudaFree -- which may synchronise the whole device --
// would stall other work.  phn_volume_averages_noalloc serves them: the
// caller passes the fields (device pointers) and the output (host struct);
// the per-block partial records of the reduction live in one fixed,
// file-scope __device__ array instead of memory allocated per call.
//
// The kernel is the fused observation pass of the leapfrog step
// (leapfrog.cu, observation-only mode), launched with one block per 32x8
// column of the lattice marching all N planes, so the number of block records
// is ceil(N/32) * ceil(N/8); the fold is finalize_averages.
#include <mutex>

#include "phn_internal.h"

namespace {

// Scratch capacity: 4096 block records of phn::REC doubles (768 KiB) plus one
// output record.  Enough for every lattice with ceil(N/32)*ceil(N/8) <= 4096,
// i.e. N <= 1024.  Every GPU that loads the library keeps this array until
// the process exits.
constexpr int kMaxBlocks = 4096;
constexpr size_t kOutOffset = (size_t)kMaxBlocks * phn::REC;  // in doubles
constexpr size_t kScratchDoubles = kOutOffset + 32;            // output record: 26 doubles

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_addr[kMaxDevices];  // device address of the array, per device

// The array's name in host code is only a host-side stand-in; the device
// address comes from cudaGetSymbolAddress, once per device, with that device
// current (it is the caller's current device here).
int scratch_address(double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return phn::cuda_error(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return phn::set_error(PHN_ERR_UNSUPPORTED, "device %d >= %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return phn::cuda_error(e, "cudaGetSymbolAddress(scratch)");
    g_scratch_addr[dev] = (double *)p;
  }
  *out = g_scratch_addr[dev];
  return PHN_OK;
}

}  // namespace

using namespace phn;

extern "C" int phn_volume_averages_noalloc(const phn_params *params, const void *d_phi, const void *d_pi,
                                           void *stream, phn_averages *out) {
  int r = validate_params(params);
  if (r) return r;
  if (params->precision == PHN_FP32_KAHAN)
    return set_error(PHN_ERR_UNSUPPORTED, "noalloc averages take plain FP64 or FP32 fields");
  const int N = params->N;
  const int gx = (N + TX - 1) / TX, gy = (N + TY - 1) / TY;
  if ((long long)gx * gy > kMaxBlocks)
    return set_error(PHN_ERR_INVALID,
                     "N=%d needs %lld scratch records; the fixed scratch holds %d (N <= 1024)", N,
                     (long long)gx * gy, kMaxBlocks);
  if (!d_phi || !d_pi || !out) return set_error(PHN_ERR_INVALID, "NULL argument");
  double *scratch = nullptr;
  r = scratch_address(&scratch);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  // the expanding box's averages at tau = T0: scale factor sqrt(1 + 2 H_0 T0)
  const Consts k0 = make_consts(params);
  const Consts k = params->expanding ? at_scale_factor(k0, sqrt(1. + 2. * params->H0 * params->T0)) : k0;
  Grid g;
  g.block = dim3(TX, TY, 1);
  g.grid = dim3(gx, gy, 1);
  g.cz = N;
  g.nblocks = gx * gy;
  // Every block overwrites its own record and finalize overwrites the output
  // record, so no scratch word is read before this call writes it: nothing
  // needs clearing.  Calls that overlap on the GPU (other streams, other host
  // threads) share the array and race; serialise them.
  const StepF s = {0.0, 0.0};
  cudaError_t e;
  if (params->precision == PHN_FP64)
    e = launch_step_f64(k, g, MODE_OBS, (const double *)d_phi, nullptr, (double *)const_cast<void *>(d_pi), s,
                        scratch, st);
  else
    e = launch_step_f32(k, g, MODE_OBS, (const float *)d_phi, nullptr, (float *)const_cast<void *>(d_pi), s,
                        scratch, st);
  if (e != cudaSuccess) return cuda_error(e, "observation kernel");
  phn_averages *d_out = (phn_averages *)(scratch + kOutOffset);
  e = launch_finalize(k, scratch, g.nblocks, d_out, st);
  if (e != cudaSuccess) return cuda_error(e, "finalize kernel");
  e = cudaMemcpyAsync(out, d_out, sizeof(phn_averages), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "averages readback");
  out->t = 0.0;
  if (out->nonfinite > 0) return set_error(PHN_ERR_NONFINITE, "%.0f non-finite field values", out->nonfinite);
  return PHN_OK;
}
