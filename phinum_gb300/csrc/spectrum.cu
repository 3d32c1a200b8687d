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
// Each mode's bin and weight are evaluated once per handle and rule into a
// 16-bit key table (bin_keys, which also counts the modes per bin), so the
// per-call pass (bin_sums) is a stream over the two half-spectra and the keys
// without FP64 square roots or divisions.  A warp takes 32 consecutive modes;
// a segmented inclusive scan over its lanes (segments = runs of equal bins)
// leaves each run's sum in the run's last lane, which adds it to the warp's
// shared-memory histogram: five shuffle steps per 32 modes however many bins
// they touch.  Accumulation is deterministic: fixed scan shape, runs that
// share a bin within a warp added in lane order, warp histograms folded per
// block in warp order, then over blocks in block order.
#include <cufft.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "float_pair.cuh"
#include "phn_internal.h"
#include "site_terms.cuh"

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
  unsigned short *keys;    // [N][N/2+1][N] bin | weight bit per mode (reference rule)
  int nblocks, nbins;
  int rblocks;             // bin_runs' grid (more, smaller blocks than bin_sums')
  double binsize;
  std::vector<int> h_counts;
  bool counts_ok;
  bool mono, u_mono;       // the key tables' rows are monotone per half (bin_runs applies)
  // density-contrast spectrum (phn_spectrum_energy), allocated on first use
  void *dfield;            // [Nc][V] Delta, then its contrast (the field's precision)
  double *dsum;            // [nblocks] per-block sums of Delta, then [nblocks] the mean
  // uniform-bin (configuration) mode, allocated on first use
  int u_nbins;
  double *u_partials, *u_bins;
  int *u_counts;
  unsigned short *u_keys;
  std::vector<int> u_h_counts;
  // device time of the last spectrum call (phn_spectrum_timing): events
  // around the transforms and around the binning of each component
  cudaEvent_t ev[3];
  bool ev_ok, pending_transform;
  double t_transform, t_binning;
};

constexpr unsigned KEY_WEIGHT2 = 0x8000u;  // the mode is counted twice (py not 0 or N/2)
constexpr unsigned KEY_BIN = 0x7fffu;

constexpr int SPEC_MAX_UNIFORM_BINS = 1024;  // per-warp histograms in shared memory
enum { RULE_REFERENCE = 0, RULE_UNIFORM = 1 };

// Lattice momentum of index n along an axis (momentumspace.cpp:222-244).
static double lattice_p(int n, int N, double a) {
  if (n < N / 2 + 1) return 2.0 / (a) * sin(n * acos(-1.) / N);
  return -2.0 / (a) * sin(n * acos(-1.) / N);
}

__device__ __forceinline__ float mag2v(float2 v) { return fmaf(v.x, v.x, v.y * v.y); }
__device__ __forceinline__ double mag2v(double2 v) { return v.x * v.x + v.y * v.y; }
__device__ __forceinline__ float dotv(float2 a, float2 b) { return fmaf(a.x, b.x, a.y * b.y); }
__device__ __forceinline__ double dotv(double2 a, double2 b) { return a.x * b.x + a.y * b.y; }

// Key of every mode of the reference's mode set, i = px + N (py + M pz) with
// px in [0,N), py in [0,N/2], pz in [0,N): the bin (bits 0-14) and the
// weight-2 bit, plus the per-bin mode counts (InitBCounts, momentumspace.cpp:
// 89-138; per-block shared-memory counts, then one global add per bin).
// rule RULE_REFERENCE: bin = int(|p| / binsize + 0.5) (momentumspace.cpp:228);
// rule RULE_UNIFORM: bin = int(|p| / binsize), binsize = p_max / nbins, the
// top edge folded into the last bin.  |p| in FP64 as the reference writes it.
__global__ void __launch_bounds__(SPEC_THREADS) bin_keys(const double *__restrict__ ptab, int N, double binsize,
                                                        int nbins, int rule, unsigned short *__restrict__ keys,
                                                        int *__restrict__ counts, int *__restrict__ flag) {
  extern __shared__ int cnt[];  // [nbins]
  for (int b = threadIdx.x; b < nbins; b += SPEC_THREADS) cnt[b] = 0;
  __syncthreads();
  const int h = N / 2, M = N / 2 + 1;
  const long long total = (long long)N * M * N;
  for (long long i = blockIdx.x * (long long)SPEC_THREADS + threadIdx.x; i < total;
       i += (long long)gridDim.x * SPEC_THREADS) {
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
    const bool two = py != 0 && py != h;
    if (bin >= nbins || bin > (int)KEY_BIN) {
      atomicOr(flag, 1);
      keys[i] = (unsigned short)KEY_BIN;
    } else {
      keys[i] = (unsigned short)(bin | (two ? KEY_WEIGHT2 : 0u));
      atomicAdd(&cnt[bin], two ? 2 : 1);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbins; b += SPEC_THREADS)
    if (cnt[b]) atomicAdd(&counts[b], cnt[b]);
}

// Per-call sums: F += w |Phi_p|^2, K += w |Pi_p|^2, Q += w Re(Phi_p Pi_p*)
// (momentumspace.cpp:222-240) for every mode, binned by its key; the
// reference's a^3 a^3 factor is applied in fold_blocks.  A mode with
// px <= N/2 is read directly from cuFFT's [pz][py][px/2+1] half-spectrum, one
// with px > N/2 from its conjugate partner (N-px, -py, -pz).  V: the scan's
// arithmetic, float for FP32 spectra, double for FP64.
// Histogram cell of the warp histograms: FP64 for FP64 spectra; for FP32
// spectra a compensated FP32 pair (Kahan: value = s - c), so that the FP32
// pass issues no FP64 instruction (GB300's FP64 rate bound it) and still
// keeps ~2^-48 of the sum.
struct CompF {
  float s, c;
};
__device__ __forceinline__ void hist_add(double &h, double v) { h += v; }
__device__ __forceinline__ void hist_add(CompF &h, float v) {
  const float y = __fsub_rn(v, h.c);
  const float t = __fadd_rn(h.s, y);
  h.c = __fsub_rn(__fsub_rn(t, h.s), y);
  h.s = t;
}
__device__ __forceinline__ double hist_value(double h) { return h; }
__device__ __forceinline__ double hist_value(CompF h) { return (double)h.s - (double)h.c; }
__device__ __forceinline__ void hist_zero(double &h) { h = 0.0; }
__device__ __forceinline__ void hist_zero(CompF &h) { h.s = h.c = 0.f; }

template <typename C, typename V>
__global__ void __launch_bounds__(SPEC_THREADS) bin_sums(const C *__restrict__ fphi, const C *__restrict__ fpi,
                                                        const unsigned short *__restrict__ keys, int N, int nbins,
                                                        double *__restrict__ partials) {
  using H = typename std::conditional<sizeof(V) == 4, CompF, double>::type;
  extern __shared__ double hist_mem[];
  H *hist = (H *)hist_mem;  // [SPEC_WARPS][3][nbins]: 8 bytes per cell either way
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < SPEC_WARPS * 3 * nbins; i += SPEC_THREADS) hist_zero(hist[i]);
  __syncthreads();
  H *hF = hist + (size_t)warp * 3 * nbins, *hK = hF + nbins, *hQ = hK + nbins;
  const unsigned full = 0xffffffffu;
  const int h = N / 2, M = N / 2 + 1;
  const int nrows = M * N;
  // a warp walks whole rows (py, pz) of the mode set, 32 px at a time: the
  // row's offsets are computed once, px comes from the lane (no 64-bit
  // division per mode); the loads of UNROLL chunks are issued together
  constexpr int UNROLL = sizeof(V) == 4 ? 4 : 2;
  for (int row = blockIdx.x * SPEC_WARPS + warp; row < nrows; row += gridDim.x * SPEC_WARPS) {
    const int py = row % M, pz = row / M;
    const long long krow = (long long)row * N;                                         // key index of px = 0
    const long long direct = ((long long)pz * N + py) * M;                              // + px, px <= N/2
    const long long mirror = ((long long)((N - pz) % N) * N + (N - py) % N) * M + N;  // - px, px > N/2
    for (int px0 = 0; px0 < N; px0 += 32 * UNROLL) {
      unsigned kk[UNROLL];
      C va[UNROLL], vb[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const int px = px0 + 32 * u + lane;
        kk[u] = 0xffffffffu;  // past the row's end
        if (px < N) {
          kk[u] = keys[krow + px];
          const long long m = px <= h ? direct + px : mirror - px;
          va[u] = fphi[m];
          vb[u] = fpi[m];
        }
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        int bin = -1;  // lanes past the end: a segment that is never written
        V f = 0, k = 0, q = 0;
        if (kk[u] != 0xffffffffu) {
          bin = (int)(kk[u] & KEY_BIN);
          f = mag2v(va[u]);
          k = mag2v(vb[u]);
          q = dotv(va[u], vb[u]);
          if (kk[u] & KEY_WEIGHT2) {  // exact doubling
            f += f;
            k += k;
            q += q;
          }
        }
        // segmented inclusive scan: a segment is a run of lanes with one bin
        const int prev = __shfl_up_sync(full, bin, 1);
        const unsigned heads = __ballot_sync(full, lane == 0 || prev != bin);
        const int start = 31 - __clz(heads & (full >> (31 - lane)));  // first lane of my segment
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const V uf = __shfl_up_sync(full, f, off), uk = __shfl_up_sync(full, k, off),
                  uq = __shfl_up_sync(full, q, off);
          if (lane - off >= start) {
            f += uf;
            k += uk;
            q += uq;
          }
        }
        // the last lane of each segment holds the segment's sum
        const int next = __shfl_down_sync(full, bin, 1);
        const bool tail = (lane == 31 || next != bin) && bin >= 0;
        const unsigned same = __match_any_sync(full, tail ? bin : -2 - lane);
        if (!__any_sync(full, tail && __popc(same) > 1)) {
          if (tail) {  // distinct bins: one update each
            hist_add(hF[bin], f);
            hist_add(hK[bin], k);
            hist_add(hQ[bin], q);
          }
        } else {  // runs sharing a bin (the mirror turn at px = N/2, a row change): in lane order
          for (unsigned tails = __ballot_sync(full, tail); tails; tails &= tails - 1) {
            if (lane == __ffs(tails) - 1) {
              hist_add(hF[bin], f);
              hist_add(hK[bin], k);
              hist_add(hQ[bin], q);
            }
            __syncwarp();
          }
        }
        __syncwarp();
      }
    }
  }
  __syncthreads();
  // fold the warp histograms in warp order; one record per block
  for (int j = threadIdx.x; j < 3 * nbins; j += SPEC_THREADS) {
    double s = 0.0;
    for (int w = 0; w < SPEC_WARPS; ++w) s += hist_value(hist[(size_t)w * 3 * nbins + j]);
    partials[(size_t)blockIdx.x * 3 * nbins + j] = s;
  }
}

// Per-call sums, FP32 spectra, by runs: the bins of a row (py, pz) are
// monotone in px on each half -- non-decreasing on [0, N/2) where |p_x|
// grows, non-increasing on [N/2, N) where it falls (checked per key table by
// keys_monotone; bin_sums serves a table that fails the check).  A warp walks
// a half row in chunks of 32 lanes x RUN_Q consecutive modes; each lane
// loads its own RUN_Q modes (keys as one 16-byte word where the edge is a
// multiple of 16, both spectra at fixed offsets from one address per lane)
// and sums the runs of equal bins in registers.  Within a chunk the bins are
// monotone, so every run has a bin no other run of the chunk has: the runs
// inside a lane's modes are staged in shared memory as they close (one
// 16-byte store, no branch around a histogram update per mode) and added to
// the warp histogram after the loop, all lanes at once; the runs that cross
// lanes join in one segmented scan per chunk (it stops at the longest
// segment), and each closes in one lane.  Each histogram cell takes at most
// one addition per chunk, in chunk order, so the sums are the same run to
// run.
constexpr int RUN_Q = 4;
constexpr int RUN_STAGE = RUN_Q - 2;  // runs strictly inside a lane's modes
constexpr int RUN_WARPS = 4;          // 128 threads: histograms of up to 1024 bins
constexpr int RUN_THREADS = 32 * RUN_WARPS;
constexpr int RUN_BLOCKS_PER_SM = 7;  // resident blocks: 71 registers, 31 KB of shared memory at 284 bins

// w2: the chunk's modes count twice (their row's py is neither 0 nor N/2,
// so the weight is one per row): the doubling of each run's sums is exact,
// and so the same bits as doubling every mode.
__device__ __forceinline__ void run_flush(CompF *hF, int nbins, int bin, float f, float k, float q, bool w2) {
  if (w2) {
    f += f;
    k += k;
    q += q;
  }
  hist_add(hF[bin], f);
  hist_add(hF[nbins + bin], k);
  hist_add(hF[2 * nbins + bin], q);
}

// One chunk of a half row: MIRROR = 0 for px in [0, N/2) (modes at
// direct + px), 1 for [N/2, N) (px = N/2 at direct + N/2, the others at
// mirror - px).
template <int MIRROR, typename I>
__device__ __forceinline__ void run_chunk(const float2 *__restrict__ fphi, const float2 *__restrict__ fpi,
                                          const unsigned short *__restrict__ keys, I krow, I direct, I mirror, int h,
                                          int c0, int x1, bool vkeys, int lane, CompF *hF, int nbins,
                                          float4 *stage) {
  const unsigned full = 0xffffffffu;
  const int cn = min(32 * RUN_Q, x1 - c0);
  const int nm = max(0, min(RUN_Q, cn - lane * RUN_Q));
  const int px0 = c0 + lane * RUN_Q;
  // the lane's modes, loaded together
  unsigned kk[RUN_Q];
  float2 va[RUN_Q], vb[RUN_Q];
  const unsigned short *pk = keys + krow + px0;
  if (vkeys && nm == RUN_Q) {  // one aligned word: krow and px0 are multiples of RUN_Q
    unsigned ww[RUN_Q / 2];
    if constexpr (RUN_Q == 8) {
      const uint4 w = *(const uint4 *)pk;
      ww[0] = w.x;
      ww[1] = w.y;
      ww[2] = w.z;
      ww[3] = w.w;
    } else {
      const uint2 w = *(const uint2 *)pk;
      ww[0] = w.x;
      ww[1] = w.y;
    }
#pragma unroll
    for (int m = 0; m < RUN_Q; m += 2) {
      kk[m] = ww[m / 2] & 0xffffu;
      kk[m + 1] = ww[m / 2] >> 16;
    }
  } else {
#pragma unroll
    for (int m = 0; m < RUN_Q; ++m) kk[m] = m < nm ? pk[m] : 0u;
  }
  const I base = MIRROR ? mirror - (I)px0 : direct + (I)px0;
  const float2 *pa = fphi + base, *pb = fpi + base;
  // the lane's RUN_Q modes are consecutive: as 16-byte words where the
  // lowest one starts on a 16-byte boundary (the row's parity, uniform per
  // warp), else one mode per load
  const I lo = MIRROR ? base - (I)(RUN_Q - 1) : base;
  if (nm == RUN_Q && (lo & 1) == 0) {
    const float4 *qa = (const float4 *)(fphi + lo), *qb = (const float4 *)(fpi + lo);
#pragma unroll
    for (int w = 0; w < RUN_Q / 2; ++w) {
      const float4 xa = qa[w], xb = qb[w];
      const int m0 = MIRROR ? RUN_Q - 1 - 2 * w : 2 * w, m1 = MIRROR ? m0 - 1 : m0 + 1;
      va[m0] = make_float2(xa.x, xa.y);
      va[m1] = make_float2(xa.z, xa.w);
      vb[m0] = make_float2(xb.x, xb.y);
      vb[m1] = make_float2(xb.z, xb.w);
    }
  } else {
#pragma unroll
    for (int m = 0; m < RUN_Q; ++m) {
      if (m < nm) {
        va[m] = MIRROR ? pa[-m] : pa[m];
        vb[m] = MIRROR ? pb[-m] : pb[m];
      }
    }
  }
  if (MIRROR && px0 == h && nm > 0) {  // px = N/2 is a direct mode
    va[0] = fphi[direct + h];
    vb[0] = fpi[direct + h];
  }
  const bool w2 = (kk[0] & KEY_WEIGHT2) != 0;  // one weight per row (lanes with modes)
  // runs of the lane's modes: the first (fb, F), the ones strictly inside
  // (staged), the last (cur, a: the whole of them when through)
  int fb = -1, cur = -1, ns = 0;
  float F0 = 0.f, F1 = 0.f, F2 = 0.f, a0 = 0.f, a1 = 0.f, a2 = 0.f;
  bool first_open = true;
#pragma unroll
  for (int m = 0; m < RUN_Q; ++m) {
    if (m < nm) {
      const float f = mag2v(va[m]), k = mag2v(vb[m]), q = dotv(va[m], vb[m]);
      const int b = (int)(kk[m] & KEY_BIN);
      const bool nw = b != cur;  // a run starts at m
      const bool close = nw && cur >= 0;
      if (close && first_open) {
        fb = cur;
        F0 = a0;
        F1 = a1;
        F2 = a2;
      }
      if (close && !first_open) stage[ns++ * 32 + lane] = make_float4(__int_as_float(cur), a0, a1, a2);
      first_open = first_open && !close;
      cur = b;
      a0 = nw ? f : a0 + f;
      a1 = nw ? k : a1 + k;
      a2 = nw ? q : a2 + q;
    }
  }
  const int lb = cur;
  const bool through = nm > 0 && first_open;
  if (through) fb = lb;
  // runs across lanes: carry C = the run through the lane's last mode
  const int lb_prev = __shfl_up_sync(full, lb, 1);
  const bool conn = lane > 0 && nm > 0 && lb_prev >= 0 && fb == lb_prev;
  const unsigned heads = __ballot_sync(full, !(through && conn));
  const int start = 31 - __clz(heads & (full >> (31 - lane)));
  // the scan stops at the first step that no lane's segment reaches back to
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    if (!__any_sync(full, lane - off >= start)) break;  // uniform per warp
    const float u0 = __shfl_up_sync(full, a0, off), u1 = __shfl_up_sync(full, a1, off),
                u2 = __shfl_up_sync(full, a2, off);
    if (lane - off >= start) {
      a0 += u0;
      a1 += u1;
      a2 += u2;
    }
  }
  const float p0 = __shfl_up_sync(full, a0, 1), p1 = __shfl_up_sync(full, a1, 1), p2 = __shfl_up_sync(full, a2, 1);
  const bool conn_next = __shfl_down_sync(full, conn, 1) && lane < 31;
  // every run of the chunk has its own bin: the closing adds touch distinct
  // cells and go in any order
  if (nm > 0 && !through) {  // the first run closes at the lane's first bin change
    if (conn) {
      F0 += p0;
      F1 += p1;
      F2 += p2;
    }
    run_flush(hF, nbins, fb, F0, F1, F2, w2);
  }
  if (nm > 0 && !conn_next) run_flush(hF, nbins, lb, a0, a1, a2, w2);
  const int nsmax = __reduce_max_sync(full, (unsigned)ns);
  for (int j = 0; j < nsmax; ++j) {
    if (j < ns) {
      const float4 v = stage[j * 32 + lane];
      run_flush(hF, nbins, __float_as_int(v.x), v.y, v.z, v.w, w2);
    }
  }
  __syncwarp();  // the histogram and the stage are read by the next chunk
}

// I: the index type of the modes, 32-bit where N^2 (N/2 + 1) fits (fewer
// registers), else 64-bit.
template <typename I>
__global__ void __launch_bounds__(RUN_THREADS, RUN_BLOCKS_PER_SM)
    bin_runs(const float2 *__restrict__ fphi, const float2 *__restrict__ fpi, const unsigned short *__restrict__ keys,
             int N, int nbins, double *__restrict__ partials) {
  extern __shared__ double run_mem[];
  CompF *hist = (CompF *)run_mem;                                      // [RUN_WARPS][3][nbins]
  float4 *stage_all = (float4 *)(run_mem + (size_t)RUN_WARPS * 3 * nbins);  // [RUN_WARPS][RUN_STAGE][32]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < RUN_WARPS * 3 * nbins; i += RUN_THREADS) hist_zero(hist[i]);
  __syncthreads();
  CompF *hF = hist + (size_t)warp * 3 * nbins;
  float4 *stage = stage_all + (size_t)warp * RUN_STAGE * 32;
  const int h = N / 2, M = N / 2 + 1;
  const int nrows = M * N;
  const bool vkeys = N % (2 * RUN_Q) == 0;  // every chunk's keys start on a RUN_Q-mode boundary
  for (int row = blockIdx.x * RUN_WARPS + warp; row < nrows; row += gridDim.x * RUN_WARPS) {
    const int py = row % M, pz = row / M;
    const I krow = (I)row * (I)N;
    const I direct = ((I)pz * (I)N + (I)py) * (I)M;
    const I mirror = ((I)((N - pz) % N) * (I)N + (I)((N - py) % N)) * (I)M + (I)N;
    for (int c0 = 0; c0 < h; c0 += 32 * RUN_Q)
      run_chunk<0, I>(fphi, fpi, keys, krow, direct, mirror, h, c0, h, vkeys, lane, hF, nbins, stage);
    for (int c0 = h; c0 < N; c0 += 32 * RUN_Q)
      run_chunk<1, I>(fphi, fpi, keys, krow, direct, mirror, h, c0, N, vkeys, lane, hF, nbins, stage);
  }
  __syncthreads();
  // the warps' cells (value s - c) fold in float pairs and widen once: the
  // grid is one wave, so every block reaches this fold at the same moment,
  // and FP64 here queued on GB300's narrow FP64 pipe
  for (int j = threadIdx.x; j < 3 * nbins; j += RUN_THREADS) {
    float sh = 0.f, sl = 0.f;
    for (int w = 0; w < RUN_WARPS; ++w) {
      const CompF c = hist[(size_t)w * 3 * nbins + j];
      fpair_add(sh, sl, c.s, -c.c);
    }
    partials[(size_t)blockIdx.x * 3 * nbins + j] = (double)sh + (double)sl;
  }
}

// Whether every row's bins are monotone on each half (bin_runs' condition):
// one thread per row and half.  Sets bit 1 of *flag on a violation.
__global__ void keys_monotone(const unsigned short *__restrict__ keys, int N, int *__restrict__ flag) {
  const int h = N / 2, M = N / 2 + 1;
  const long long n = 2LL * M * N;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const long long row = t >> 1;
    const int half = (int)(t & 1);
    const unsigned short *k = keys + row * N;
    int prev = half ? 0x7fffffff : -1;
    bool ok = true;
    for (int px = half ? h : 0; px < (half ? N : h); ++px) {
      const int b = (int)(k[px] & KEY_BIN);
      if (half ? b > prev : b < prev) ok = false;
      prev = b;
    }
    if (!ok) atomicOr(flag, 2);
  }
}

// The per-bin totals over the blocks' partials: one block per entry (F, K, Q
// of a bin), a strided sum per thread and a fixed tree, so the result does
// not depend on timing.
__global__ void __launch_bounds__(256) fold_blocks(const double *__restrict__ partials, int nblocks, int nbins,
                                                   double scale, double *__restrict__ out) {
  __shared__ double sh[256];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += 256) s += partials[(size_t)b * 3 * nbins + j];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[j] = sh[0] * scale;
}

// Delta of component a at every site (site_delta: kinetic, the full squared
// forward differences, Delta's potential), into out[], and per block the FP64
// sum of the block's values (each thread's values summed in FP32 pairs
// first).  A thread walks sites i = t, t + T, ... of the grid's T threads.
template <typename T, bool KAHAN>
__global__ void __launch_bounds__(SPEC_THREADS) delta_field(const T *__restrict__ phi, const float *__restrict__ cphi,
                                                           const T *__restrict__ pi, const float *__restrict__ cpi,
                                                           int N, const Consts k, T *__restrict__ out,
                                                           double *__restrict__ bsum) {
  using A = typename std::conditional<std::is_same<T, float>::value, float, double>::type;
  const size_t NN = (size_t)N * N, V = NN * N;
  A hi = 0, lo = 0;
  for (size_t i = blockIdx.x * (size_t)SPEC_THREADS + threadIdx.x; i < V; i += (size_t)gridDim.x * SPEC_THREADS) {
    const int z = (int)(i / NN), y = (int)((i - (size_t)z * NN) / N), x = (int)(i - (size_t)z * NN - (size_t)y * N);
    const A d = site_delta<A, KAHAN>(phi, cphi, pi, cpi, N, x, y, z, k);
    out[i] = (T)d;
    const A t = hi + d, bb = t - hi;  // TwoSum
    lo += (hi - (t - bb)) + (d - bb);
    hi = t;
  }
  __shared__ double sh[SPEC_THREADS];
  sh[threadIdx.x] = (double)hi + (double)lo;
  __syncthreads();
  for (int w = SPEC_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < (unsigned)w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] += sh[0];
}

// Aavden = (sum of Delta over every component and site) / N^3
// (momentumspace.cpp:165-176), in a fixed order; into *mean.
__global__ void delta_mean(const double *__restrict__ bsum, int nblocks, int N, double *__restrict__ mean) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += bsum[b];
    *mean = s / ((double)N * (double)N * (double)N);
  }
}

// The density contrast (Delta - Aavden) / Aavden in the field's precision
// (momentumspace.cpp:177-181).
template <typename T>
__global__ void delta_contrast(T *__restrict__ f, size_t n, const double *__restrict__ mean) {
  const T m = (T)*mean;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    T v = f[i];
    v -= m;
    v /= m;
    f[i] = v;
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
  cudaFree(s->keys);
  cudaFree(s->u_partials);
  cudaFree(s->u_bins);
  cudaFree(s->u_counts);
  cudaFree(s->u_keys);
  cudaFree(s->dfield);
  cudaFree(s->dsum);
  if (s->ev_ok)
    for (int j = 0; j < 3; ++j) cudaEventDestroy(s->ev[j]);
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

static size_t n_modes(int N) { return (size_t)N * (N / 2 + 1) * N; }

// Key table and mode counts of one rule (bin_keys), counts copied to host.
static int build_keys(phn_handle *h, unsigned short *keys, int *counts, int nbins, double binsize, int rule,
                      std::vector<int> &h_counts, bool *mono) {
  SpecState *s = (SpecState *)h->spec;
  cudaError_t e = cudaMemsetAsync(counts, 0, nbins * sizeof(int), h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->flag, 0, sizeof(int), h->stream);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemsetAsync");
  bin_keys<<<s->nblocks, SPEC_THREADS, nbins * sizeof(int), h->stream>>>(s->ptab, h->p.N, binsize, nbins, rule, keys,
                                                                          counts, s->flag);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "bin_keys");
  keys_monotone<<<s->nblocks, SPEC_THREADS, 0, h->stream>>>(keys, h->p.N, s->flag);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "keys_monotone");
  h->launches += 2;
  h_counts.resize(nbins);
  int flag = 0;
  e = cudaMemcpyAsync(h_counts.data(), counts, nbins * sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, s->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_error(e, "mode counts");
  if (flag & 1) return set_error(PHN_ERR_INVALID, "bin array too small (momentumspace.cpp:128)");
  *mono = (flag & 2) == 0;
  return PHN_OK;
}

// Shared memory of bin_runs: the warp histograms, then the warps' stages of
// runs inside a lane (16 bytes each).
static size_t run_smem(int nbins) {
  return (size_t)RUN_WARPS * 3 * nbins * sizeof(double) + (size_t)RUN_WARPS * RUN_STAGE * 32 * sizeof(float4);
}

static int spec_init(phn_handle *h) {
  if (h->spec) return PHN_OK;
  SpecState *s = new SpecState();
  h->spec = s;
  const int N = h->p.N;
  bin_geometry(h->p, &s->nbins, &s->binsize);
  s->nblocks = 152 * 4;
  s->rblocks = 152 * RUN_BLOCKS_PER_SM;
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
  CKS(cudaMalloc(&s->partials, (size_t)std::max(s->nblocks, s->rblocks) * 3 * s->nbins * sizeof(double)));
  CKS(cudaMalloc(&s->bins, (size_t)3 * s->nbins * sizeof(double)));
  CKS(cudaMalloc(&s->counts, (size_t)s->nbins * sizeof(int)));
  CKS(cudaMalloc(&s->flag, sizeof(int)));
  CKS(cudaMalloc(&s->keys, n_modes(N) * sizeof(unsigned short)));
  for (int j = 0; j < 3; ++j) CKS(cudaEventCreate(&s->ev[j]));
  s->ev_ok = true;
  std::vector<double> tab(N);
  for (int n = 0; n < N; ++n) tab[n] = lattice_p(n, N, h->p.a);
  CKS(cudaMemcpy(s->ptab, tab.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  if (cufftPlan3d(&s->plan, N, N, N, dbl ? CUFFT_D2Z : CUFFT_R2C) != CUFFT_SUCCESS)
    return set_error(PHN_ERR_CUDA, "cufftPlan3d(%d^3) failed", N);
  s->plan_ok = true;
  if (cufftSetStream(s->plan, h->stream) != CUFFT_SUCCESS) return set_error(PHN_ERR_CUDA, "cufftSetStream failed");
  // the largest histogram either rule uses
  const int maxb = s->nbins > SPEC_MAX_UNIFORM_BINS ? s->nbins : SPEC_MAX_UNIFORM_BINS;
  const size_t smem_max = (size_t)SPEC_WARPS * 3 * maxb * sizeof(double);
  CKS(cudaFuncSetAttribute(bin_sums<float2, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
  CKS(cudaFuncSetAttribute(bin_sums<double2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
  CKS(cudaFuncSetAttribute(bin_keys, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(maxb * sizeof(int))));
  CKS(cudaFuncSetAttribute(bin_runs<unsigned>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)run_smem(maxb)));
  CKS(cudaFuncSetAttribute(bin_runs<size_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)run_smem(maxb)));
#undef CKS
  // keys and mode counts of the reference rule (InitBCounts): field independent
  return build_keys(h, s->keys, s->counts, s->nbins, s->binsize, RULE_REFERENCE, s->h_counts, &s->mono);
}

// One component: R2C of phi and pi, the binned sums, the three bin arrays
// into hb ([3][nbins], scaled by a^3 a^3).
static int bin_spectra(phn_handle *h, const void *fa, const void *fb, const unsigned short *keys, int nbins,
                       double *partials, double *bins, double scale, bool mono, std::vector<double> &hb);

static int spectrum_component(phn_handle *h, int a, const unsigned short *keys, int nbins, double *partials,
                              double *bins, double scale, bool mono, std::vector<double> &hb) {
  SpecState *s = (SpecState *)h->spec;
  const bool dbl = h->p.precision == PHN_FP64;
  cufftResult fr;
  cudaEventRecord(s->ev[0], h->stream);
  s->pending_transform = true;  // bin_spectra adds the transforms' time
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
  return bin_spectra(h, s->fphi, s->fpi, keys, nbins, partials, bins, scale, mono, hb);
}

// The binned sums of two half-spectra (F from the first, K from the second,
// Q from both) into hb ([3][nbins], scaled).
static int bin_spectra(phn_handle *h, const void *fa, const void *fb, const unsigned short *keys, int nbins,
                       double *partials, double *bins, double scale, bool mono, std::vector<double> &hb) {
  SpecState *s = (SpecState *)h->spec;
  const int N = h->p.N;
  const bool dbl = h->p.precision == PHN_FP64;
  const size_t smem = (size_t)SPEC_WARPS * 3 * nbins * sizeof(double);
  const bool transformed = s->pending_transform;  // spectrum_component recorded ev[0]
  s->pending_transform = false;
  cudaEventRecord(s->ev[1], h->stream);
  if (dbl)
    bin_sums<double2, double><<<s->nblocks, SPEC_THREADS, smem, h->stream>>>(
        (const double2 *)fa, (const double2 *)fb, keys, N, nbins, partials);
  else if (mono)
    (n_modes(N) < ((size_t)1 << 31) ? bin_runs<unsigned> : bin_runs<size_t>)<<<s->rblocks, RUN_THREADS,
                                                                                  run_smem(nbins), h->stream>>>(
        (const float2 *)fa, (const float2 *)fb, keys, N, nbins, partials);
  else
    bin_sums<float2, float><<<s->nblocks, SPEC_THREADS, smem, h->stream>>>(
        (const float2 *)fa, (const float2 *)fb, keys, N, nbins, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "bin_sums");
  fold_blocks<<<3 * nbins, 256, 0, h->stream>>>(partials, (!dbl && mono) ? s->rblocks : s->nblocks, nbins, scale,
                                                  bins);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "fold_blocks");
  h->launches += 2;
  cudaEventRecord(s->ev[2], h->stream);
  hb.resize((size_t)3 * nbins);
  e = cudaMemcpyAsync(hb.data(), bins, hb.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_error(e, "spectrum readback");
  float ms = 0.f;
  if (transformed && cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]) == cudaSuccess) s->t_transform += ms;
  if (cudaEventElapsedTime(&ms, s->ev[1], s->ev[2]) == cudaSuccess) s->t_binning += ms;
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
  s->t_transform = s->t_binning = 0.0;
  s->pending_transform = false;
  if (nbins < s->nbins) return set_error(PHN_ERR_TRUNCATED, "nbins=%d < %d", nbins, s->nbins);
  const int Nc = h->p.Nc;
  const double f3 = (h->p.a * h->p.a) * h->p.a;  // fftXtoP_direct's a^3 (clusterfft.cpp:187,222)
  std::vector<double> hb;
  for (int k = 0; k < s->nbins * Nc; ++k) {
    if (F) F[k] = 0.0;
    if (K) K[k] = 0.0;
    if (Q) Q[k] = 0.0;
  }
  for (int a = 0; a < Nc; ++a) {
    r = spectrum_component(h, a, s->keys, s->nbins, s->partials, s->bins, f3 * f3, s->mono, hb);
    if (r) return r;
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

int phn_spectrum_timing(const phn_handle *h, double *transform_ms, double *binning_ms) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  const SpecState *s = (const SpecState *)h->spec;
  if (!s) return set_error(PHN_ERR_INVALID, "no spectrum call on this handle");
  if (transform_ms) *transform_ms = s->t_transform;
  if (binning_ms) *binning_ms = s->t_binning;
  return PHN_OK;
}

int phn_spectrum_energy(phn_handle *h, double *D, int *counts, int nbins) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (h->p.potential < 2)
    return set_error(PHN_ERR_UNSUPPORTED, "Delta has no form for theory %d (the reference's withEnergyPS build "
                     "compiles for theories 2-5)", h->p.potential);
  int r = spec_init(h);
  if (r) {
    spectrum_release(h);
    return r;
  }
  SpecState *s = (SpecState *)h->spec;
  s->t_transform = s->t_binning = 0.0;
  s->pending_transform = false;
  if (nbins < s->nbins) return set_error(PHN_ERR_TRUNCATED, "nbins=%d < %d", nbins, s->nbins);
  const int N = h->p.N, Nc = h->p.Nc;
  const bool dbl = h->p.precision == PHN_FP64;
  const size_t V = h->V, esize = dbl ? sizeof(double) : sizeof(float);
  cudaStream_t st = h->stream;
  cudaError_t e = cudaSuccess;
  if (!s->dfield) {
    e = cudaMalloc(&s->dfield, (size_t)Nc * V * esize);
    if (e == cudaSuccess) e = cudaMalloc(&s->dsum, (size_t)(s->nblocks + 1) * sizeof(double));
    if (e != cudaSuccess) {
      cudaFree(s->dfield);
      s->dfield = nullptr;
      return cuda_error(e, "energy spectrum buffers");
    }
  }
  // Delta of every component, its mean over them all, the contrast
  const Consts k = consts_now(h);
  const bool kahan = h->p.precision == PHN_FP32_KAHAN;
  e = cudaMemsetAsync(s->dsum, 0, (size_t)s->nblocks * sizeof(double), st);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemsetAsync");
  for (int a = 0; a < Nc; ++a) {
    const size_t o = (size_t)a * V;
    if (dbl)
      delta_field<double, false><<<s->nblocks, SPEC_THREADS, 0, st>>>(
          (const double *)h->phi[h->cur] + o, nullptr, (const double *)h->pi + o, nullptr, N, k,
          (double *)s->dfield + o, s->dsum);
    else if (kahan)
      delta_field<float, true><<<s->nblocks, SPEC_THREADS, 0, st>>>(
          (const float *)h->phi[h->cur] + o, h->cphi + o, (const float *)h->pi + o, h->cpi + o, N, k,
          (float *)s->dfield + o, s->dsum);
    else
      delta_field<float, false><<<s->nblocks, SPEC_THREADS, 0, st>>>(
          (const float *)h->phi[h->cur] + o, nullptr, (const float *)h->pi + o, nullptr, N, k,
          (float *)s->dfield + o, s->dsum);
  }
  double *mean = s->dsum + s->nblocks;
  delta_mean<<<1, 32, 0, st>>>(s->dsum, s->nblocks, N, mean);
  if (dbl)
    delta_contrast<double><<<s->nblocks, SPEC_THREADS, 0, st>>>((double *)s->dfield, (size_t)Nc * V, mean);
  else
    delta_contrast<float><<<s->nblocks, SPEC_THREADS, 0, st>>>((float *)s->dfield, (size_t)Nc * V, mean);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "Delta kernels");
  h->launches += Nc + 2;
  // per component: R2C of the contrast and its binned power (the F sum of
  // the binning with the same spectrum in both slots)
  const double f3 = (h->p.a * h->p.a) * h->p.a;
  std::vector<double> hb;
  for (int a = 0; a < Nc; ++a) {
    const size_t o = (size_t)a * V;
    cufftResult fr;
    if (dbl)
      fr = cufftExecD2Z(s->plan, (double *)s->dfield + o, (cufftDoubleComplex *)s->fphi);
    else
      fr = cufftExecR2C(s->plan, (float *)s->dfield + o, (cufftComplex *)s->fphi);
    if (fr != CUFFT_SUCCESS) return set_error(PHN_ERR_CUDA, "cuFFT exec failed (%d)", (int)fr);
    r = bin_spectra(h, s->fphi, s->fphi, s->keys, s->nbins, s->partials, s->bins, f3 * f3, s->mono, hb);
    if (r) return r;
    for (int b = 0; b < s->nbins; ++b)
      if (D) D[b * Nc + a] = hb[b];
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
  s->t_transform = s->t_binning = 0.0;
  s->pending_transform = false;
  const int N = h->p.N, Nc = h->p.Nc;
  // p_max = pTmax of momentumspace.cpp:43, the largest lattice |p|
  const double pmax = sqrt(3.0 * (4.0 / (h->p.a * h->p.a)));
  if (s->u_nbins != nbins) {
    cudaFree(s->u_partials);
    cudaFree(s->u_bins);
    cudaFree(s->u_counts);
    cudaFree(s->u_keys);
    s->u_partials = s->u_bins = nullptr;
    s->u_counts = nullptr;
    s->u_keys = nullptr;
    s->u_nbins = 0;
    cudaError_t e = cudaMalloc(&s->u_partials, (size_t)std::max(s->nblocks, s->rblocks) * 3 * nbins * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->u_bins, (size_t)3 * nbins * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->u_counts, (size_t)nbins * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&s->u_keys, n_modes(N) * sizeof(unsigned short));
    if (e != cudaSuccess) return cuda_error(e, "uniform spectrum buffers");
    r = build_keys(h, s->u_keys, s->u_counts, nbins, pmax / nbins, RULE_UNIFORM, s->u_h_counts, &s->u_mono);
    if (r) return r;
    s->u_nbins = nbins;
  }
  const double f3 = (h->p.a * h->p.a) * h->p.a;
  std::vector<double> hb;
  for (int a = 0; a < Nc; ++a) {
    r = spectrum_component(h, a, s->u_keys, nbins, s->u_partials, s->u_bins, f3 * f3, s->u_mono, hb);
    if (r) return r;
    for (int b = 0; b < nbins; ++b) {
      if (F) F[b * Nc + a] = hb[b];
      if (K) K[b * Nc + a] = hb[nbins + b];
      if (Q) Q[b * Nc + a] = hb[2 * nbins + b];
    }
  }
  if (counts)
    for (int b = 0; b < nbins; ++b) counts[b] = s->u_h_counts[b];
  return PHN_OK;
}

}  // extern "C"
