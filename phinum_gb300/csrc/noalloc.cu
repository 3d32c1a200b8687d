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
#include <cuda.h>
#include <cudaTypedefs.h>

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

// The device address of the array belongs to the CUDA context the module was
// loaded into.  A device reset (cudaDeviceReset, by this or another runtime in
// the process) or a context the host created with the driver API gives the
// same device another context, in which the old address means nothing.  So
// the address is cached per device together with the unique ID of the context
// it was looked up in (cuCtxGetId: IDs are never reused in a process), and
// looked up again when the calling thread's current context has another ID.
constexpr int kMaxDevices = 64;
struct ScratchSlot {
  unsigned long long ctx_id;  // 0: no set-up on this device yet
  double *addr;
};
std::mutex g_mu;
ScratchSlot g_slot[kMaxDevices];

// cuCtxGetCurrent / cuCtxGetId from the driver through the runtime (the
// library does not link libcuda); null when the driver lacks them, and then
// every call looks the address up.
PFN_cuCtxGetCurrent_v4000 g_ctx_current = nullptr;
PFN_cuCtxGetId_v12000 g_ctx_id = nullptr;
std::once_flag g_entry_once;

void load_entry_points() {
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    g_ctx_current = (PFN_cuCtxGetCurrent_v4000)fn;
  fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    g_ctx_id = (PFN_cuCtxGetId_v12000)fn;
}

// ID of the context current on the calling thread; 0 when none is current yet
// (a fresh thread, or right after a reset) or the driver cannot tell.
unsigned long long current_context_id() {
  if (!g_ctx_current || !g_ctx_id) return 0;
  CUcontext c = nullptr;
  if (g_ctx_current(&c) != CUDA_SUCCESS || !c) return 0;
  unsigned long long id = 0;
  if (g_ctx_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// The array's name in host code is only a host-side stand-in; the device
// address comes from cudaGetSymbolAddress, with the device current (it is the
// caller's current device here), at set-up: the first call on a device, and
// again whenever that device's context has changed since.
int scratch_address(double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return phn::cuda_error(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return phn::set_error(PHN_ERR_UNSUPPORTED, "device %d >= %d", dev, kMaxDevices);
  std::call_once(g_entry_once, load_entry_points);
  std::lock_guard<std::mutex> lock(g_mu);
  ScratchSlot &s = g_slot[dev];
  const unsigned long long now = current_context_id();
  if (s.addr && now != 0 && now == s.ctx_id) {
    *out = s.addr;
    return PHN_OK;
  }
  // set-up (this also makes the runtime's context current when none was)
  void *p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return phn::cuda_error(e, "cudaGetSymbolAddress(scratch)");
  s.addr = (double *)p;
  s.ctx_id = current_context_id();
  *out = s.addr;
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
  out->t = params->T0;  // the state is taken as the one at tau = T0, as a fresh handle stamps it
  if (out->nonfinite > 0) return set_error(PHN_ERR_NONFINITE, "%.0f non-finite field values", out->nonfinite);
  return PHN_OK;
}
