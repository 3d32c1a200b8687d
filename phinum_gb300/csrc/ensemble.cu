// Batched ensemble: many independent lattices of uneven sizes evolved by one
// persistent kernel per step, the step loop captured in a CUDA graph.
//
// Replaces running the reference once per realization (one `main` per seed).
// All members share the clock (a, dt, T0) -- the kick/drift factors of a step
// are the same for every member -- and may differ in N (multiples of 32),
// potential and couplings.  Fields live back to back in one FP32 buffer.
//
// Work list: items = (member, 32-wide x tile, TY-row y tile, CZ-plane z
// chunk), member-major; or, for the x4 tiles, (member, chunk of 128 W
// consecutive plane sites, CZ-plane z chunk) with four x-sites per thread.  A persistent grid (SMs x resident blocks) walks the
// list round-robin; every item is the same size (32 x TY x CZ sites), so the
// load is balanced whatever the mix of lattice sizes.  The per-site arithmetic
// is kick_drift_f32 (kick.cuh), the same bits as the single-lattice kernels,
// so a member's fields equal those of a single run exactly.  The tile shape
// (TY, CZ) is chosen by phn_ensemble_autotune, which times the candidates on
// the live ensemble.  Steps run in chunks of kGraphSteps captured once as a
// CUDA graph; the chunk's kick/drift factors are read from a device table
// refilled before each launch, so one graph serves the whole run.
#include <math.h>
#include <string.h>

#include <vector>

#include "kick.cuh"
#include "observe.cuh"
#include "phn_internal.h"

namespace phn {

struct EnsMember {
  int N;
  int theory;
  long long off;  // element offset of the member in the ensemble buffers
  Consts k;
};

struct EnsItem {
  int member, x0, y0, z0, nz;
};

// ty: rows per block (scalar tiles) or warps per block (x4 tiles).
struct EnsTile {
  int ty, cz;
  bool x4;
};
constexpr EnsTile kEnsTiles[] = {{8, 16, false}, {4, 16, false}, {8, 8, false}, {4, 32, false},
                                 {8, 32, false}, {4, 8, false},  {8, 16, true},  {4, 16, true},
                                 {8, 32, true},  {4, 32, true},  {2, 32, true}};
constexpr int kNumEnsTiles = 11;
constexpr int kGraphSteps = 50;

// The FP32 couplings of theories 0 and 1 at scale factor sf, for an
// expanding member: the fields of at_scale_factor (api.cu) that the FP32 kick
// and observation read, by the same FP64 expressions, so that a member gets
// the bits a single lattice gets (dynamics.cpp:88-104, fieldanalysis.cpp:
// 461-615).  Once per work item: a few FP64 operations against the item's
// thousands of sites.
__device__ __forceinline__ void couplings_at(Consts &k, double sf) {
  k.sf = sf;
  k.mmM_f = (float)(k.mmM * sf * sf);
  k.h_f = (float)(k.h * sf * sf * sf);
  k.mmh_f = (float)(k.mm_half_M * sf * sf);
  if (k.theory == 0) {
    k.c6_f = (float)(1.0 / (k.kappa * k.kappa * k.c120 * sf * sf));
    k.e6_f = (float)(1.0 / (k.c720 * sf * sf));
  }
  k.hub_f = (float)(k.H0 / sf);
}

// factors: [3 per step] kick factor, drift factor, the kick's scale factor;
// sf_obs: the scale factor of an observation (MODE_OBS).
template <int TY, int MODE>
__global__ void __launch_bounds__(32 * TY) ens_step(const EnsMember *__restrict__ members,
                                                    const EnsItem *__restrict__ items, int nitems,
                                                    const float *__restrict__ phi, float *__restrict__ phi_out,
                                                    float *__restrict__ pi, const double *__restrict__ factors,
                                                    int slot, double sf_obs, double *__restrict__ partials) {
  const float fk = MODE == MODE_OBS ? 0.f : (float)factors[3 * slot];
  const float fd = MODE == MODE_OBS ? 0.f : (float)factors[3 * slot + 1];
  const double sf = MODE == MODE_OBS ? sf_obs : factors[3 * slot + 2];
  const int tid = threadIdx.x + 32 * threadIdx.y;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const EnsItem I = items[it];
    const int N = members[I.member].N;
    const int theory = members[I.member].theory;
    const long long off = members[I.member].off;
    Consts k = members[I.member].k;
    if (k.expansion) couplings_at(k, sf);  // uniform per item
    const float *f = phi + off;
    float *fo = phi_out + off;
    float *pp = pi + off;
    const size_t NN = (size_t)N * N;
    const int x = I.x0 + threadIdx.x, y = I.y0 + threadIdx.y;
    const int xp = (x + 1 == N) ? 0 : x + 1, xm = (x == 0) ? N - 1 : x - 1;
    const int yp = (y + 1 == N) ? 0 : y + 1, ym = (y == 0) ? N - 1 : y - 1;
    const size_t col = (size_t)y * N + x;
    const int z0 = I.z0, z1 = I.z0 + I.nz;
    AccF accf;
    if (MODE != MODE_STEP) accf.init();
    float cm = __ldg(f + (size_t)((z0 == 0) ? N - 1 : z0 - 1) * NN + col);
    float c = __ldg(f + (size_t)z0 * NN + col);
    for (int z = z0; z < z1; ++z) {
      const int zn = (z + 1 == N) ? 0 : z + 1;
      const size_t pl = (size_t)z * NN;
      const float cp = __ldg(f + (size_t)zn * NN + col);
      const float fxp = __ldg(f + pl + (size_t)y * N + xp);
      const float fxm = __ldg(f + pl + (size_t)y * N + xm);
      const float fyp = __ldg(f + pl + (size_t)yp * N + x);
      const float fym = __ldg(f + pl + (size_t)ym * N + x);
      const float p = pp[pl + col];
      if (MODE != MODE_STEP) {
        const float c1[1] = {c}, p1[1] = {p}, x1[1] = {fxp}, y1[1] = {fyp}, z1v[1] = {cp};
        const long long kidx = (long long)(col + (size_t)(z + 1) * NN);
        if (theory == 0)
          observe_f32<1, 0>(accf, k, c1, p1, x1, y1, z1v, kidx);
        else
          observe_f32<1, 1>(accf, k, c1, p1, x1, y1, z1v, kidx);
      }
      if (MODE != MODE_OBS) {
        float pn, fn;
        if (theory == 0)
          kick_drift_f32<0>(k, fk, fd, c, fxm, fxp, fym, fyp, cm, cp, p, pn, fn);
        else
          kick_drift_f32<1>(k, fk, fd, c, fxm, fxp, fym, fyp, cm, cp, p, pn, fn);
        pp[pl + col] = pn;
        fo[pl + col] = fn;
      }
      cm = c;
      c = cp;
    }
    if (MODE != MODE_STEP) {
      Acc acc;
      accf.to_double(acc);
      block_store_n(acc, partials, tid, TY, (size_t)it);
    }
  }
}

// Four consecutive x-sites per thread (16-byte loads and stores); a warp
// covers 128 consecutive sites of a plane -- several rows when N < 128 -- and
// a block W warps.  An item's chunk starts at plane site q0 = y0 * N + x0.
// x neighbours inside the thread's four sites come from registers, the two
// outside ones from scalar loads (the same cache lines as the neighbouring
// lanes' vectors); y rows and z planes are float4.  kick_drift_f32 gets the
// same values as in the scalar kernels, so the fields are bit-identical.
template <int W, int MODE>
__global__ void __launch_bounds__(32 * W) ens_step_x4(const EnsMember *__restrict__ members,
                                                      const EnsItem *__restrict__ items, int nitems,
                                                      const float *__restrict__ phi, float *__restrict__ phi_out,
                                                      float *__restrict__ pi, const double *__restrict__ factors,
                                                      int slot, double sf_obs, double *__restrict__ partials) {
  const float fk = MODE == MODE_OBS ? 0.f : (float)factors[3 * slot];
  const float fd = MODE == MODE_OBS ? 0.f : (float)factors[3 * slot + 1];
  const double sf = MODE == MODE_OBS ? sf_obs : factors[3 * slot + 2];
  const int tid = threadIdx.x + 32 * threadIdx.y;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const EnsItem I = items[it];
    const int N = members[I.member].N;
    const int theory = members[I.member].theory;
    const long long off = members[I.member].off;
    Consts k = members[I.member].k;
    if (k.expansion) couplings_at(k, sf);  // uniform per item
    const float *f = phi + off;
    float *fo = phi_out + off;
    float *pp = pi + off;
    const int NN = N * N;
    const int q = I.y0 * N + I.x0 + 4 * tid;  // this thread's first site in the plane
    const int y = q / N, x = q - y * N;
    const int qxl = (x == 0) ? q + N - 1 : q - 1;
    const int qxr = (x + 4 == N) ? q + 4 - N : q + 4;
    const int qyp = (y + 1 == N) ? q - (N - 1) * N : q + N;
    const int qym = (y == 0) ? q + (N - 1) * N : q - N;
    const int z0 = I.z0, z1 = I.z0 + I.nz;
    AccF accf;
    if (MODE != MODE_STEP) accf.init();
    float4 cm = __ldg((const float4 *)(f + (size_t)((z0 == 0) ? N - 1 : z0 - 1) * NN + q));
    float4 c = __ldg((const float4 *)(f + (size_t)z0 * NN + q));
    for (int z = z0; z < z1; ++z) {
      const int zn = (z + 1 == N) ? 0 : z + 1;
      const float *pl = f + (size_t)z * NN;
      const size_t i = (size_t)z * NN + q;
      const float4 cp = __ldg((const float4 *)(f + (size_t)zn * NN + q));
      const float4 yp = __ldg((const float4 *)(pl + qyp));
      const float4 ym = __ldg((const float4 *)(pl + qym));
      const float xm = __ldg(pl + qxl), xp = __ldg(pl + qxr);
      const float4 p = *(const float4 *)(pp + i);
      if (MODE != MODE_STEP) {
        const float cv[4] = {c.x, c.y, c.z, c.w}, pv[4] = {p.x, p.y, p.z, p.w};
        const float xv[4] = {c.y, c.z, c.w, xp}, yv[4] = {yp.x, yp.y, yp.z, yp.w};
        const float zv[4] = {cp.x, cp.y, cp.z, cp.w};
        const long long kidx = (long long)q + (long long)(z + 1) * NN;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (theory == 0)
            observe_f32<1, 0>(accf, k, cv + e, pv + e, xv + e, yv + e, zv + e, kidx + e);
          else
            observe_f32<1, 1>(accf, k, cv + e, pv + e, xv + e, yv + e, zv + e, kidx + e);
        }
      }
      if (MODE != MODE_OBS) {
        float4 pn, fn;
        if (theory == 0) {
          kick_drift_f32<0>(k, fk, fd, c.x, xm, c.y, ym.x, yp.x, cm.x, cp.x, p.x, pn.x, fn.x);
          kick_drift_f32<0>(k, fk, fd, c.y, c.x, c.z, ym.y, yp.y, cm.y, cp.y, p.y, pn.y, fn.y);
          kick_drift_f32<0>(k, fk, fd, c.z, c.y, c.w, ym.z, yp.z, cm.z, cp.z, p.z, pn.z, fn.z);
          kick_drift_f32<0>(k, fk, fd, c.w, c.z, xp, ym.w, yp.w, cm.w, cp.w, p.w, pn.w, fn.w);
        } else {
          kick_drift_f32<1>(k, fk, fd, c.x, xm, c.y, ym.x, yp.x, cm.x, cp.x, p.x, pn.x, fn.x);
          kick_drift_f32<1>(k, fk, fd, c.y, c.x, c.z, ym.y, yp.y, cm.y, cp.y, p.y, pn.y, fn.y);
          kick_drift_f32<1>(k, fk, fd, c.z, c.y, c.w, ym.z, yp.z, cm.z, cp.z, p.z, pn.z, fn.z);
          kick_drift_f32<1>(k, fk, fd, c.w, c.z, xp, ym.w, yp.w, cm.w, cp.w, p.w, pn.w, fn.w);
        }
        *(float4 *)(pp + i) = pn;
        *(float4 *)(fo + i) = fn;
      }
      cm = c;
      c = cp;
    }
    if (MODE != MODE_STEP) {
      Acc acc;
      accf.to_double(acc);
      block_store_n(acc, partials, tid, W, (size_t)it);
    }
  }
}

// One block per member folds that member's item records, in item order.
__global__ void __launch_bounds__(FIN_THREADS) ens_fold(const double *__restrict__ partials,
                                                        const int *__restrict__ item_begin,
                                                        const EnsMember *__restrict__ members, double sf_obs,
                                                        phn_averages *__restrict__ out) {
  const int m = blockIdx.x;
  Consts k = members[m].k;
  if (k.expansion) k.sf = sf_obs;  // the fold's expanding-box terms read H0 / sf
  fold_records(partials, item_begin[m], item_begin[m + 1], k, out + m);
}

template <int TY, int MODE>
static cudaError_t ens_launch_t(int grid, const EnsMember *members, const EnsItem *items, int nitems, const float *phi,
                                float *phi_out, float *pi, const double *factors, int slot, double sf_obs,
                                double *partials, cudaStream_t st) {
  ens_step<TY, MODE><<<grid, dim3(32, TY), 0, st>>>(members, items, nitems, phi, phi_out, pi, factors, slot, sf_obs,
                                                    partials);
  return cudaGetLastError();
}

template <int W, int MODE>
static cudaError_t ens_launch_x4_t(int grid, const EnsMember *members, const EnsItem *items, int nitems,
                                   const float *phi, float *phi_out, float *pi, const double *factors, int slot,
                                   double sf_obs, double *partials, cudaStream_t st) {
  ens_step_x4<W, MODE><<<grid, dim3(32, W), 0, st>>>(members, items, nitems, phi, phi_out, pi, factors, slot, sf_obs,
                                                     partials);
  return cudaGetLastError();
}

static cudaError_t ens_launch(const EnsTile &T, int mode, int grid, const EnsMember *members, const EnsItem *items,
                              int nitems, const float *phi, float *phi_out, float *pi, const double *factors,
                              int slot, double sf_obs, double *partials, cudaStream_t st) {
  const int ty = T.ty;
  if (T.x4) {
#define PHN_ENS4(WV, MD) \
  return ens_launch_x4_t<WV, MD>(grid, members, items, nitems, phi, phi_out, pi, factors, slot, sf_obs, partials, st)
    if (ty == 8) {
      if (mode == MODE_STEP) PHN_ENS4(8, MODE_STEP);
      if (mode == MODE_STEP_OBS) PHN_ENS4(8, MODE_STEP_OBS);
      PHN_ENS4(8, MODE_OBS);
    }
    if (ty == 4) {
      if (mode == MODE_STEP) PHN_ENS4(4, MODE_STEP);
      if (mode == MODE_STEP_OBS) PHN_ENS4(4, MODE_STEP_OBS);
      PHN_ENS4(4, MODE_OBS);
    }
    if (mode == MODE_STEP) PHN_ENS4(2, MODE_STEP);
    if (mode == MODE_STEP_OBS) PHN_ENS4(2, MODE_STEP_OBS);
    PHN_ENS4(2, MODE_OBS);
#undef PHN_ENS4
  }
#define PHN_ENS(TYV, MD) \
  return ens_launch_t<TYV, MD>(grid, members, items, nitems, phi, phi_out, pi, factors, slot, sf_obs, partials, st)
  if (ty == 8) {
    if (mode == MODE_STEP) PHN_ENS(8, MODE_STEP);
    if (mode == MODE_STEP_OBS) PHN_ENS(8, MODE_STEP_OBS);
    PHN_ENS(8, MODE_OBS);
  }
  if (mode == MODE_STEP) PHN_ENS(4, MODE_STEP);
  if (mode == MODE_STEP_OBS) PHN_ENS(4, MODE_STEP_OBS);
  PHN_ENS(4, MODE_OBS);
#undef PHN_ENS
}

static int ens_grid(const EnsTile &T) {
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void *fn;
  if (T.x4)
    fn = T.ty == 8 ? (const void *)ens_step_x4<8, MODE_STEP>
                   : (T.ty == 4 ? (const void *)ens_step_x4<4, MODE_STEP> : (const void *)ens_step_x4<2, MODE_STEP>);
  else
    fn = T.ty == 8 ? (const void *)ens_step<8, MODE_STEP> : (const void *)ens_step<4, MODE_STEP>;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 32 * T.ty, 0) != cudaSuccess || occ < 1) occ = 1;
  return sms * occ;
}

}  // namespace phn

using namespace phn;

struct phn_ensemble {
  int n;
  std::vector<phn_params> p;
  std::vector<long long> off;
  std::vector<size_t> V;
  size_t total;
  int maxN;
  EnsMember *d_members;
  float *phi[2];
  float *pi;
  int cur;
  // tiles
  int tile;
  EnsItem *d_items;
  int nitems;
  int *d_item_begin;  // [n+1]
  int grid;
  double *partials;
  int partial_cap;
  phn_averages *d_avg;
  // clock shared by all members (dynamics.cpp:28-50); the expanding box's
  // conformal times and scale factor (dynamics.cpp:196-213)
  double tau, dtau, last_mom, last_field;
  bool expanding;
  double H0, tau_c, sf, last_mom_c, last_field_c;
  int steps;
  // factor table and graph
  double *d_factors;   // [3 * kGraphSteps]: kick, drift, the kick's scale factor
  double *h_factors;   // pinned, grows
  size_t h_factors_cap;
  cudaGraphExec_t graph[2];  // by the parity of cur at launch
  bool graph_ok[2];
  cudaStream_t stream;
  cudaEvent_t ev0, ev1;
  long long launches;
  double last_ms;
  int last_steps;
  double *d_ref;
  phn_handle view;  // island labelling of one member through the handle path
};

static void ens_free_graphs(phn_ensemble *e) {
  for (int i = 0; i < 2; ++i)
    if (e->graph_ok[i]) {
      cudaGraphExecDestroy(e->graph[i]);
      e->graph_ok[i] = false;
    }
}

static void ens_free(phn_ensemble *e) {
  if (!e) return;
  ens_free_graphs(e);
  islands_release(&e->view);
  cudaFree(e->d_members);
  cudaFree(e->phi[0]);
  cudaFree(e->phi[1]);
  cudaFree(e->pi);
  cudaFree(e->d_items);
  cudaFree(e->d_item_begin);
  cudaFree(e->partials);
  cudaFree(e->d_avg);
  cudaFree(e->d_factors);
  cudaFree(e->d_ref);
  if (e->h_factors) cudaFreeHost(e->h_factors);
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

#define CKE(call)                                        \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_error(e_, #call); \
  } while (0)

// Builds the member-major work list for tile configuration t.
static int ens_set_tile(phn_ensemble *e, int t) {
  const EnsTile T = kEnsTiles[t];
  std::vector<EnsItem> items;
  std::vector<int> begin(e->n + 1);
  for (int m = 0; m < e->n; ++m) {
    begin[m] = (int)items.size();
    const int N = e->p[m].N;
    const int cz = T.cz < N ? T.cz : N;
    if (T.x4) {
      // chunks of 128 W plane sites; N a multiple of 32 makes N^2 a multiple
      // of 1024, so chunks tile every plane exactly
      const int chunk = 128 * T.ty, NN = N * N;
      for (int z0 = 0; z0 < N; z0 += cz)
        for (int q0 = 0; q0 < NN; q0 += chunk) {
          EnsItem I = {m, q0 % N, q0 / N, z0, (z0 + cz <= N) ? cz : N - z0};
          items.push_back(I);
        }
      continue;
    }
    for (int z0 = 0; z0 < N; z0 += cz)
      for (int y0 = 0; y0 < N; y0 += T.ty)
        for (int x0 = 0; x0 < N; x0 += 32) {
          EnsItem I = {m, x0, y0, z0, (z0 + cz <= N) ? cz : N - z0};
          items.push_back(I);
        }
  }
  begin[e->n] = (int)items.size();
  cudaFree(e->d_items);
  e->d_items = nullptr;
  CKE(cudaMalloc(&e->d_items, items.size() * sizeof(EnsItem)));
  CKE(cudaMemcpy(e->d_items, items.data(), items.size() * sizeof(EnsItem), cudaMemcpyHostToDevice));
  CKE(cudaMemcpy(e->d_item_begin, begin.data(), begin.size() * sizeof(int), cudaMemcpyHostToDevice));
  e->nitems = (int)items.size();
  if (e->nitems > e->partial_cap) {
    cudaFree(e->partials);
    e->partials = nullptr;
    CKE(cudaMalloc(&e->partials, (size_t)e->nitems * REC * sizeof(double)));
    e->partial_cap = e->nitems;
  }
  e->tile = t;
  e->grid = ens_grid(T);
  ens_free_graphs(e);
  return PHN_OK;
}

static int ens_launch_step(phn_ensemble *e, int mode, int slot, int cur) {
  CKE(ens_launch(kEnsTiles[e->tile], mode, e->grid, e->d_members, e->d_items, e->nitems, e->phi[cur],
                 e->phi[1 - cur], e->pi, e->d_factors, slot, e->sf, e->partials, e->stream));
  e->launches++;
  return PHN_OK;
}

// Captures kGraphSteps plain steps starting from buffer parity `cur`.
static int ens_build_graph(phn_ensemble *e, int cur) {
  if (e->graph_ok[cur]) return PHN_OK;
  cudaGraph_t g;
  CKE(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  int c = cur, r = PHN_OK;
  for (int i = 0; i < kGraphSteps && r == PHN_OK; ++i) {
    r = ens_launch_step(e, MODE_STEP, i, c);
    c = 1 - c;
  }
  cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
  if (r) return r;
  if (ce != cudaSuccess) return cuda_error(ce, "cudaStreamEndCapture");
  e->launches -= kGraphSteps;  // counted when the graph runs
  ce = cudaGraphInstantiate(&e->graph[cur], g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) return cuda_error(ce, "cudaGraphInstantiate");
  e->graph_ok[cur] = true;
  return PHN_OK;
}

// The expanding box's conformal time and scale factor at tau (the handle's
// clock, dynamics.cpp:28-50).
static void ens_conformal(phn_ensemble *e) {
  e->tau_c = (sqrt(1. + 2. * e->H0 * e->tau) - 1.) / e->H0;
  e->sf = sqrt(1. + 2. * e->H0 * e->tau);
}

// Host clock for one step (dynamics.cpp:196-237, as the handle's step):
// writes f[0] the kick factor, f[1] the drift factor (conformal-time
// differences in the expanding box), f[2] the scale factor of the kick.
static void ens_clock_step(phn_ensemble *e, double *f) {
  e->tau += 0.5 * e->dtau;
  if (e->expanding) {
    ens_conformal(e);
    f[0] = e->tau_c - e->last_mom_c;
    f[2] = e->sf;
  } else {
    f[0] = e->tau - e->last_mom;
    f[2] = 1.0;
  }
  e->last_mom = e->tau;
  e->last_mom_c = e->expanding ? e->tau_c : e->tau;
  e->tau += 0.5 * e->dtau;
  if (e->expanding) {
    ens_conformal(e);
    f[1] = e->tau_c - e->last_field_c;
  } else {
    f[1] = e->tau - e->last_field;
    e->tau_c = e->tau;
  }
  e->last_field = e->tau;
  e->last_field_c = e->tau_c;
  e->steps++;
}

extern "C" {

int phn_ensemble_create(const phn_params *members, int n, phn_ensemble **out) {
  if (!out || !members || n < 1) return set_error(PHN_ERR_INVALID, "bad argument");
  *out = nullptr;
  for (int m = 0; m < n; ++m) {
    int r = validate_params(&members[m]);
    if (r) return r;
    const phn_params &q = members[m];
    if (q.precision != PHN_FP32 || q.Nc != 1 || q.N % 32 != 0 || q.potential > 1)
      return set_error(PHN_ERR_UNSUPPORTED,
                       "member %d: ensembles take FP32, Nc = 1, N a multiple of 32, theory 0 or 1", m);
    if (q.a != members[0].a || q.dt != members[0].dt || q.T0 != members[0].T0 ||
        (q.expanding != 0) != (members[0].expanding != 0) || (q.expanding && q.H0 != members[0].H0))
      return set_error(PHN_ERR_INVALID, "member %d: members share a, dt, T0 and the box (expanding, H0): one clock",
                       m);
  }
  phn_ensemble *e = new phn_ensemble();
  e->n = n;
  e->p.assign(members, members + n);
  std::vector<EnsMember> hm(n);
  size_t total = 0;
  e->maxN = 0;
  for (int m = 0; m < n; ++m) {
    const size_t V = (size_t)members[m].N * members[m].N * members[m].N;
    e->V.push_back(V);
    e->off.push_back((long long)total);
    hm[m].N = members[m].N;
    hm[m].theory = members[m].potential;
    hm[m].off = (long long)total;
    hm[m].k = make_consts(&members[m]);
    total += V;
    if (members[m].N > e->maxN) e->maxN = members[m].N;
  }
  e->total = total;
  cudaError_t ce;
#define CKC(call)                                 \
  do {                                            \
    ce = (call);                                  \
    if (ce != cudaSuccess) {                      \
      int rr = cuda_error(ce, #call);             \
      ens_free(e);                                \
      return rr;                                  \
    }                                             \
  } while (0)
  CKC(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
  CKC(cudaEventCreate(&e->ev0));
  CKC(cudaEventCreate(&e->ev1));
  CKC(cudaMalloc(&e->d_members, n * sizeof(EnsMember)));
  CKC(cudaMemcpy(e->d_members, hm.data(), n * sizeof(EnsMember), cudaMemcpyHostToDevice));
  CKC(cudaMalloc(&e->phi[0], total * sizeof(float)));
  CKC(cudaMalloc(&e->phi[1], total * sizeof(float)));
  CKC(cudaMalloc(&e->pi, total * sizeof(float)));
  CKC(cudaMemset(e->phi[0], 0, total * sizeof(float)));
  CKC(cudaMemset(e->phi[1], 0, total * sizeof(float)));
  CKC(cudaMemset(e->pi, 0, total * sizeof(float)));
  CKC(cudaMalloc(&e->d_item_begin, (n + 1) * sizeof(int)));
  CKC(cudaMalloc(&e->d_avg, n * sizeof(phn_averages)));
  CKC(cudaMalloc(&e->d_factors, 3 * kGraphSteps * sizeof(double)));
  const size_t refn = (size_t)e->maxN * e->maxN * (e->maxN + 2);
  CKC(cudaMalloc(&e->d_ref, refn * sizeof(double)));
#undef CKC
  int r = ens_set_tile(e, 0);
  if (r) {
    ens_free(e);
    return r;
  }
  *out = e;
  return phn_ensemble_reset(e);
}

int phn_ensemble_destroy(phn_ensemble *e) {
  if (!e) return PHN_OK;
  cudaStreamSynchronize(e->stream);
  ens_free(e);
  return PHN_OK;
}

int phn_ensemble_reset(phn_ensemble *e) {
  if (!e) return set_error(PHN_ERR_INVALID, "ensemble is NULL");
  e->tau = e->p[0].T0;
  e->dtau = e->p[0].dt * e->p[0].a;
  e->last_mom = e->last_field = e->tau;
  e->expanding = e->p[0].expanding != 0;
  e->H0 = e->p[0].H0;
  if (e->expanding) {
    ens_conformal(e);
  } else {
    e->tau_c = e->tau;
    e->sf = 1.0;
  }
  e->last_mom_c = e->last_field_c = e->tau_c;
  e->steps = 0;
  return PHN_OK;
}

int phn_ensemble_upload(phn_ensemble *e, int m, const double *Phi, const double *Pi) {
  if (!e || m < 0 || m >= e->n || !Phi || !Pi) return set_error(PHN_ERR_INVALID, "bad argument");
  const int N = e->p[m].N;
  const size_t n = (size_t)N * N * (N + 2);
  CKE(cudaMemcpyAsync(e->d_ref, Phi, n * sizeof(double), cudaMemcpyHostToDevice, e->stream));
  CKE(launch_from_ref(e->d_ref, e->phi[e->cur] + e->off[m], PHN_FP32, N, 1, e->stream));
  CKE(cudaMemcpyAsync(e->d_ref, Pi, n * sizeof(double), cudaMemcpyHostToDevice, e->stream));
  CKE(launch_from_ref(e->d_ref, e->pi + e->off[m], PHN_FP32, N, 1, e->stream));
  e->launches += 2;
  CKE(cudaStreamSynchronize(e->stream));
  return PHN_OK;
}

int phn_ensemble_download(phn_ensemble *e, int m, double *Phi, double *Pi) {
  if (!e || m < 0 || m >= e->n || (!Phi && !Pi)) return set_error(PHN_ERR_INVALID, "bad argument");
  const int N = e->p[m].N;
  const size_t slab = (size_t)N * N, n = slab * (N + 2);
  if (Phi) {
    CKE(launch_to_ref(e->phi[e->cur] + e->off[m], e->d_ref, PHN_FP32, N, 1, e->stream));
    CKE(cudaMemcpyAsync(Phi, e->d_ref, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    CKE(cudaStreamSynchronize(e->stream));
  }
  if (Pi) {
    CKE(launch_to_ref(e->pi + e->off[m], e->d_ref, PHN_FP32, N, 1, e->stream));
    CKE(cudaMemcpyAsync(Pi + slab, e->d_ref + slab, slab * N * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    CKE(cudaStreamSynchronize(e->stream));
  }
  return PHN_OK;
}

int phn_ensemble_evolve(phn_ensemble *e, int nsteps) {
  if (!e || nsteps < 0) return set_error(PHN_ERR_INVALID, "bad argument");
  if ((size_t)3 * nsteps > e->h_factors_cap) {
    if (e->h_factors) cudaFreeHost(e->h_factors);
    e->h_factors = nullptr;
    e->h_factors_cap = 3 * (size_t)(nsteps + kGraphSteps);
    CKE(cudaHostAlloc((void **)&e->h_factors, e->h_factors_cap * sizeof(double), cudaHostAllocDefault));
  }
  // the whole call's factors are written before any copy reads them
  for (int s = 0; s < nsteps; ++s) ens_clock_step(e, &e->h_factors[3 * s]);
  CKE(cudaEventRecord(e->ev0, e->stream));
  int done = 0;
  while (nsteps - done >= kGraphSteps) {
    int r = ens_build_graph(e, e->cur);
    if (r) return r;
    CKE(cudaMemcpyAsync(e->d_factors, e->h_factors + 3 * done, 3 * kGraphSteps * sizeof(double),
                        cudaMemcpyHostToDevice, e->stream));
    CKE(cudaGraphLaunch(e->graph[e->cur], e->stream));
    e->launches += kGraphSteps;
    done += kGraphSteps;  // kGraphSteps is even: the buffer parity is unchanged
  }
  if (done < nsteps) {
    const int rest = nsteps - done;
    CKE(cudaMemcpyAsync(e->d_factors, e->h_factors + 3 * done, 3 * rest * sizeof(double), cudaMemcpyHostToDevice,
                        e->stream));
    for (int i = 0; i < rest; ++i) {
      int r = ens_launch_step(e, MODE_STEP, i, e->cur);
      if (r) return r;
      e->cur = 1 - e->cur;
    }
  }
  CKE(cudaEventRecord(e->ev1, e->stream));
  CKE(cudaEventSynchronize(e->ev1));
  float ms = 0.f;
  CKE(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
  e->last_ms = ms;
  e->last_steps = nsteps;
  return PHN_OK;
}

int phn_ensemble_averages(phn_ensemble *e, phn_averages *out) {
  if (!e || !out) return set_error(PHN_ERR_INVALID, "bad argument");
  int r = ens_launch_step(e, MODE_OBS, 0, e->cur);
  if (r) return r;
  ens_fold<<<e->n, FIN_THREADS, 0, e->stream>>>(e->partials, e->d_item_begin, e->d_members, e->sf, e->d_avg);
  CKE(cudaGetLastError());
  e->launches++;
  CKE(cudaMemcpyAsync(out, e->d_avg, e->n * sizeof(phn_averages), cudaMemcpyDeviceToHost, e->stream));
  CKE(cudaStreamSynchronize(e->stream));
  int nonfinite = 0;
  for (int m = 0; m < e->n; ++m) {
    out[m].t = e->tau;
    if (out[m].nonfinite > 0) nonfinite = 1;
  }
  if (nonfinite) return set_error(PHN_ERR_NONFINITE, "non-finite field values in a member");
  return PHN_OK;
}

int phn_ensemble_islands(phn_ensemble *e, int m, double thres, int mode, int z_periodic, int *labels,
                         phn_island *out, int max_out, int *n_islands) {
  if (!e || m < 0 || m >= e->n) return set_error(PHN_ERR_INVALID, "bad argument");
  phn_handle &v = e->view;
  if (v.p.N != e->p[m].N) islands_release(&v);  // the label buffers are sized per lattice
  v.p = e->p[m];
  v.k = make_consts(&e->p[m]);
  v.V = e->V[m];
  v.elem = sizeof(float);
  v.cur = 0;
  v.phi[0] = e->phi[e->cur] + e->off[m];
  v.pi = e->pi + e->off[m];
  v.stream = e->stream;
  v.tau = e->tau;  // the expanding box's island terms read the scale factor
  v.tau_c = e->tau_c;
  v.sf = e->sf;
  const int r = phn_islands(&v, thres, mode, z_periodic, labels, out, max_out, n_islands);
  e->launches += v.launches;
  v.launches = 0;
  return r;
}

int phn_ensemble_autotune(phn_ensemble *e, int steps, int *tile, double *best_ms) {
  if (!e || steps < 1) return set_error(PHN_ERR_INVALID, "bad argument");
  // pi is updated in place by a step: keep a copy and restore it after each
  // trial (phi[cur] is only read), so tuning leaves the ensemble unchanged
  float *save = nullptr;
  CKE(cudaMallocAsync((void **)&save, e->total * sizeof(float), e->stream));
  CKE(cudaMemcpyAsync(save, e->pi, e->total * sizeof(float), cudaMemcpyDeviceToDevice, e->stream));
  const double f[3] = {e->dtau, e->dtau, e->sf};
  CKE(cudaMemcpyAsync(e->d_factors, f, sizeof(f), cudaMemcpyHostToDevice, e->stream));
  double best = 1e30;
  int best_t = e->tile;
  for (int round = 0; round < 2; ++round)
    for (int t = 0; t < kNumEnsTiles; ++t) {
      int r = ens_set_tile(e, t);
      if (r) return r;
      for (int i = 0; i < steps + 2; ++i) {
        if (i == 2) CKE(cudaEventRecord(e->ev0, e->stream));
        r = ens_launch_step(e, MODE_STEP, 0, e->cur);
        if (r) return r;
      }
      CKE(cudaEventRecord(e->ev1, e->stream));
      CKE(cudaEventSynchronize(e->ev1));
      float ms = 0.f;
      CKE(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
      CKE(cudaMemcpyAsync(e->pi, save, e->total * sizeof(float), cudaMemcpyDeviceToDevice, e->stream));
      if (ms / steps < best) {
        best = ms / steps;
        best_t = t;
      }
    }
  CKE(cudaFreeAsync(save, e->stream));
  int r = ens_set_tile(e, best_t);
  if (r) return r;
  CKE(cudaStreamSynchronize(e->stream));
  if (tile) *tile = best_t;
  if (best_ms) *best_ms = best;
  return PHN_OK;
}

int phn_ensemble_set_tile(phn_ensemble *e, int tile) {
  if (!e || tile < 0 || tile >= kNumEnsTiles) return set_error(PHN_ERR_INVALID, "bad argument");
  return ens_set_tile(e, tile);
}

int phn_ensemble_stats(const phn_ensemble *e, long long *launches, double *last_ms, int *last_steps) {
  if (!e) return set_error(PHN_ERR_INVALID, "ensemble is NULL");
  if (launches) *launches = e->launches;
  if (last_ms) *last_ms = e->last_ms;
  if (last_steps) *last_steps = e->last_steps;
  return PHN_OK;
}

int phn_ensemble_time(const phn_ensemble *e, double *tau, int *steps) {
  if (!e) return set_error(PHN_ERR_INVALID, "ensemble is NULL");
  if (tau) *tau = e->tau;
  if (steps) *steps = e->steps;
  return PHN_OK;
}

}  // extern "C"
