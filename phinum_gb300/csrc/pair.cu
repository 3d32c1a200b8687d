// Leapfrog in FP32 pairs: double-float arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2
// (about 48 significant bits).  Additions use Knuth's TwoSum for the high
// words and add the low words into the error (the "sloppy" double-float sum),
// products use the FMA error of the high words (Dekker's product with an
// FMA, T. J. Dekker, Numer. Math. 18, 1971; Knuth, TAOCP vol. 2, 4.2.2), and
// every result is renormalised with Fast2Sum.  GB300's FP64 rate is a small
// fraction of its FP32 rate; a pair step costs about 110 FP32 operations per
// site.  On a 32^3 phi^6 run of 1000 steps its phi is 1.7e-6 (relative L2)
// from FP64's, against 4.7e-5 for plain FP32: the trajectory differences of a
// chaotic field grow over the run, and the pair's come mostly from the
// Laplacian's high-word differences (see pair_force_w).
//
// It serves the adjoint's forward solve: the sigmoid objective amplifies a
// change of the final state some 400-fold into the gradient, and compensated
// FP32 does not help there, because the increments dt F and dt pi are
// themselves rounded to FP32 every step (an error correlated from step to
// step, which grows linearly).  Here force, increments and updates are all
// pair arithmetic.  Theories 0 and 1, Nc = 1, static or expanding box.
#include "phn_internal.h"

namespace phn {

struct F2 {
  float hi, lo;
};

__device__ __forceinline__ F2 f2_fast(float s, float e) {  // Fast2Sum, |s| >= |e|
  F2 r;
  r.hi = __fadd_rn(s, e);
  r.lo = __fsub_rn(e, __fsub_rn(r.hi, s));
  return r;
}

__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return f2_fast(s, e);
}

__device__ __forceinline__ F2 f2_neg(F2 a) { return F2{-a.hi, -a.lo}; }

__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return f2_fast(p, e);
}

// c + a b with one renormalisation: the FMA error of the high words'
// product and the TwoSum error of c.hi + p add into one error term (15 FP32
// operations, against 18 for f2_mul then f2_add; about 10% further from FP64
// on a 32^3 phi^6 run of 1000 steps).
__device__ __forceinline__ F2 f2_madd(F2 c, F2 a, F2 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float pe = __fmaf_rn(a.hi, b.hi, -p);
  const float s = __fadd_rn(c.hi, p);
  const float bb = __fsub_rn(s, c.hi);
  float e = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  e = __fadd_rn(e, __fadd_rn(c.lo, pe));
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return f2_fast(s, e);
}

// c + a b where |c| >= |a b| is the rule (the drift phi + dt pi; c4 + l c6):
// Fast2Sum instead of TwoSum for the high words (12 operations).  Where the
// rule fails -- phi near a zero crossing -- the sum keeps the rounding of the
// larger term, an FP32-level error at that site and step; on a 32^3 phi^6 run
// of 1000 steps phi ends 1.6x further from FP64 (2.6e-6 relative) than with
// TwoSum everywhere.
__device__ __forceinline__ F2 f2_madd_dom(F2 c, F2 a, F2 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float pe = __fmaf_rn(a.hi, b.hi, -p);
  const float s = __fadd_rn(c.hi, p);
  float e = __fsub_rn(p, __fsub_rn(s, c.hi));
  e = __fadd_rn(e, __fadd_rn(c.lo, pe));
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return f2_fast(s, e);
}

// a^2: the FMA error of hi^2 plus the cross term 2 hi lo.
__device__ __forceinline__ F2 f2_sqr(F2 a) {
  const float p = __fmul_rn(a.hi, a.hi);
  float e = __fmaf_rn(a.hi, a.hi, -p);
  e = __fmaf_rn(__fadd_rn(a.hi, a.hi), a.lo, e);
  return f2_fast(p, e);
}

// The pair of a double: hi = RN(x), lo = RN(x - hi).
__host__ __device__ inline F2 f2_of(double x) {
  F2 r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}

// Per-launch constants: the kick's coefficients as pairs.
struct PairConsts {
  int N, theory;
  int a2_pow2;                // 1/a^2 is a power of two: the Laplacian scales exactly
  F2 inv_a2, mmM, c4, c6, h;  // 1/a^2, Mass_Mode M^2, Lambda_Mode/(6 Nc), 1/(120 Nc^2 Kappa^2), h
  F2 fk, fd;                  // kick and drift factors of this step
};

// Lap(phi) - V'(phi) from the neighbour-difference sum s:
// V' = (mmM + l (c4 + l c6)) phi (+ h), l = phi^2, in fused pair
// multiply-adds.
__device__ __forceinline__ F2 pair_potential_force(const PairConsts &k, F2 c, F2 s) {
  const F2 lap = k.a2_pow2 ? F2{__fmul_rn(s.hi, k.inv_a2.hi), __fmul_rn(s.lo, k.inv_a2.hi)} : f2_mul(s, k.inv_a2);
  const F2 l = f2_sqr(c);
  F2 coef = k.c4;
  if (k.theory == 0) coef = f2_madd_dom(k.c4, l, k.c6);
  coef = f2_madd(k.mmM, coef, l);
  F2 f = f2_madd(lap, f2_neg(coef), c);
  if (k.theory == 1) f = f2_add(f, f2_neg(k.h));
  return f;
}

// F = Lap(phi) - V'(phi), V' = (mmM + l (c4 + l c6)) phi (+ h), l = phi^2;
// the Laplacian as the sum of the six neighbour differences (each a pair
// difference: exact in its high words even where phi changes sign between
// neighbours).
__device__ __forceinline__ F2 pair_force(const PairConsts &k, F2 c, const F2 nb[6]) {
  const F2 mc = f2_neg(c);
  F2 s = f2_add(nb[0], mc);
#pragma unroll
  for (int j = 1; j < 6; ++j) s = f2_add(s, f2_add(nb[j], mc));
  return pair_potential_force(k, c, s);
}

// The same force with the Laplacian's six differences taken word by word:
// the high words of neighbouring sites subtract exactly (Sterbenz) wherever
// phi keeps its sign between them and their differences add plainly (small
// numbers on one grid of ulps: exact unless the partial sums outgrow it), the
// low words' differences add plainly, and one TwoSum joins the two.  Against
// a TwoSum per high-word difference this is 5x further from FP64 on a 32^3
// phi^6 run of 1000 steps (1.7e-6 against 3.3e-7 relative in phi; FP32:
// 4.7e-5) for 30 fewer operations per site: the adjoint's gradient error
// stays well inside its 1e-4 target.
__device__ __forceinline__ F2 pair_force_w(const PairConsts &k, F2 c, const F2 nb[6]) {
  float acc = 0.f, lo = 0.f;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    acc = __fadd_rn(acc, __fsub_rn(nb[j].hi, c.hi));
    lo = __fadd_rn(lo, __fsub_rn(nb[j].lo, c.lo));
  }
  const float sh = __fadd_rn(acc, lo), bb = __fsub_rn(sh, acc);  // TwoSum(acc, lo)
  const F2 s = F2{sh, __fadd_rn(__fsub_rn(acc, __fsub_rn(sh, bb)), __fsub_rn(lo, bb))};
  return pair_potential_force(k, c, s);
}

// Four consecutive x-sites per thread, one plane: pi += fk F(phi) in place,
// phi' = phi + fd pi'.  Both words of phi and pi move as float4; the x
// neighbours outside the four come as scalars.  N a multiple of 4.
template <int XS>
struct PairVec;
template <>
struct PairVec<4> {
  using T = float4;
  __device__ static void unpack(const T &v, float *o) {
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
  }
  __device__ static T pack(const float *o) { return make_float4(o[0], o[1], o[2], o[3]); }
};
template <>
struct PairVec<2> {
  using T = float2;
  __device__ static void unpack(const T &v, float *o) {
    o[0] = v.x;
    o[1] = v.y;
  }
  __device__ static T pack(const float *o) { return make_float2(o[0], o[1]); }
};

// XS consecutive x-sites per thread (4: float4 words, 2: float2), one plane
// per thread; a warp covers 32 XS sites of a row.
template <int XS>
__global__ void __launch_bounds__(256, XS == 4 ? 4 : 1) step_pair_xs(const PairConsts k, const float *__restrict__ ph,
                                                                  const float *__restrict__ pl,
                                                                  float *__restrict__ qh, float *__restrict__ ql,
                                                                  float *__restrict__ oh, float *__restrict__ ol) {
  using PV = PairVec<XS>;
  using V = typename PV::T;
  const int N = k.N;
  const int x0 = XS * (blockIdx.x * 32 + threadIdx.x), y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
  if (x0 >= N || y >= N) return;
  const size_t NN = (size_t)N * N;
  const size_t plane = (size_t)z * NN, row = plane + (size_t)y * N;
  const size_t i = row + x0;
  const size_t iyp = plane + (size_t)(y + 1 == N ? 0 : y + 1) * N + x0;
  const size_t iym = plane + (size_t)(y == 0 ? N - 1 : y - 1) * N + x0;
  const size_t izp = (size_t)(z + 1 == N ? 0 : z + 1) * NN + (size_t)y * N + x0;
  const size_t izm = (size_t)(z == 0 ? N - 1 : z - 1) * NN + (size_t)y * N + x0;
  const size_t ixl = row + (x0 == 0 ? N - 1 : x0 - 1), ixr = row + (x0 + XS == N ? 0 : x0 + XS);
  auto ld = [](const float *f, size_t j) { return *(const V *)(f + j); };
  float chv[XS], clv[XS], yphv[XS], yplv[XS], ymhv[XS], ymlv[XS], zphv[XS], zplv[XS], zmhv[XS], zmlv[XS], qhv[XS],
      qlv[XS];
  PV::unpack(ld(ph, i), chv);
  PV::unpack(ld(pl, i), clv);
  PV::unpack(ld(ph, iyp), yphv);
  PV::unpack(ld(pl, iyp), yplv);
  PV::unpack(ld(ph, iym), ymhv);
  PV::unpack(ld(pl, iym), ymlv);
  PV::unpack(ld(ph, izp), zphv);
  PV::unpack(ld(pl, izp), zplv);
  PV::unpack(ld(ph, izm), zmhv);
  PV::unpack(ld(pl, izm), zmlv);
  const F2 xl = F2{ph[ixl], pl[ixl]}, xr = F2{ph[ixr], pl[ixr]};
  PV::unpack(ld(qh, i), qhv);
  PV::unpack(ld(ql, i), qlv);
  float nqh[XS], nql[XS], nph[XS], npl[XS];
#pragma unroll
  for (int j = 0; j < XS; ++j) {
    const F2 c = F2{chv[j], clv[j]};
    const F2 left = j == 0 ? xl : F2{chv[j - 1], clv[j - 1]};
    const F2 right = j == XS - 1 ? xr : F2{chv[j + 1], clv[j + 1]};
    const F2 nb[6] = {right, left, F2{yphv[j], yplv[j]}, F2{ymhv[j], ymlv[j]}, F2{zphv[j], zplv[j]},
                      F2{zmhv[j], zmlv[j]}};
    const F2 f = pair_force_w(k, c, nb);
    const F2 q = f2_madd(F2{qhv[j], qlv[j]}, f, k.fk);
    const F2 p = f2_madd_dom(c, q, k.fd);
    nqh[j] = q.hi;
    nql[j] = q.lo;
    nph[j] = p.hi;
    npl[j] = p.lo;
  }
  *(V *)(qh + i) = PV::pack(nqh);
  *(V *)(ql + i) = PV::pack(nql);
  *(V *)(oh + i) = PV::pack(nph);
  *(V *)(ol + i) = PV::pack(npl);
}

// One leapfrog step on pairs: pi += fk F(phi) in place, phi' = phi + fd pi'.
// Block (32, 8) covers 32 x-sites by 8 y-rows; each thread marches cz planes
// of one (x, y) column with phi(z-1), phi(z), phi(z+1) in registers.
__global__ void __launch_bounds__(256) step_pair(const PairConsts k, int cz, const float *__restrict__ ph,
                                                 const float *__restrict__ pl, float *__restrict__ qh,
                                                 float *__restrict__ ql, float *__restrict__ oh,
                                                 float *__restrict__ ol) {
  const int N = k.N;
  const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  if (x >= N || y >= N) return;
  const int z0 = blockIdx.z * cz, z1 = min(N, z0 + cz);
  const size_t NN = (size_t)N * N;
  const int xp = x + 1 == N ? 0 : x + 1, xm = x == 0 ? N - 1 : x - 1;
  const int yp = y + 1 == N ? 0 : y + 1, ym = y == 0 ? N - 1 : y - 1;
  const size_t col = (size_t)y * N + x;
  auto at = [&](size_t i) { return F2{ph[i], pl[i]}; };
  const int zm0 = z0 == 0 ? N - 1 : z0 - 1;
  F2 below = at((size_t)zm0 * NN + col), c = at((size_t)z0 * NN + col);
  for (int z = z0; z < z1; ++z) {
    const size_t plane = (size_t)z * NN;
    const int zp = z + 1 == N ? 0 : z + 1;
    const F2 above = at((size_t)zp * NN + col);
    const F2 nb[6] = {at(plane + (size_t)y * N + xp), at(plane + (size_t)y * N + xm),
                      at(plane + (size_t)yp * N + x), at(plane + (size_t)ym * N + x), above, below};
    const F2 f = pair_force(k, c, nb);
    const size_t i = plane + col;
    F2 q = F2{qh[i], ql[i]};
    q = f2_madd(q, f, k.fk);
    qh[i] = q.hi;
    ql[i] = q.lo;
    const F2 p = f2_madd_dom(c, q, k.fd);
    oh[i] = p.hi;
    ol[i] = p.lo;
    below = c;
    c = above;
  }
}

// Reference layout (FP64, ghosts) -> pairs of the [z][y][x] interior, and
// pairs -> FP64 [z][y][x].
__global__ void pair_from_ref(const double *__restrict__ ref, float *__restrict__ hi, float *__restrict__ lo,
                              size_t V, size_t slab) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < V; i += (size_t)gridDim.x * blockDim.x) {
    const F2 v = f2_of(ref[slab + i]);
    hi[i] = v.hi;
    lo[i] = v.lo;
  }
}

__global__ void pair_to_f64(const float *__restrict__ hi, const float *__restrict__ lo, double *__restrict__ out,
                            size_t V) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < V; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (double)hi[i] + (double)lo[i];
}

PairConsts pair_consts(const Consts &k) {
  PairConsts c;
  c.N = k.N;
  c.theory = k.theory;
  c.inv_a2 = f2_of(1.0 / k.a2);
  {
    int ex = 0;
    c.a2_pow2 = c.inv_a2.lo == 0.f && frexp((double)c.inv_a2.hi, &ex) == 0.5 && ex > -100 && ex < 100;
  }
  c.mmM = f2_of(k.mmM);
  c.c4 = f2_of(k.lm / k.six_nc);
  // the expanding box's couplings at the step's scale factor: mmM and h come
  // scaled (at_scale_factor), c6 is divided by sf^2 here (sf = 1 when static)
  c.c6 = f2_of(k.theory == 0 ? 1.0 / (k.kappa * k.kappa * k.c120 * k.sf * k.sf) : 0.0);
  c.h = f2_of(k.h);
  c.fk = c.fd = F2{0.f, 0.f};
  return c;
}

constexpr int PAIR_CZ = 16;

cudaError_t launch_step_pair(const Consts &k, double fk, double fd, const float *ph, const float *pl, float *qh,
                             float *ql, float *oh, float *ol, cudaStream_t st) {
  PairConsts c = pair_consts(k);
  c.fk = f2_of(fk);
  c.fd = f2_of(fd);
  const int N = k.N;
  // four sites per thread where rows hold whole float4 words; two (float2)
  // measured 22% slower at 128^3 (more loads per site), so they serve only
  // edges that are even but not multiples of 4
  if (N % 4 == 0) {  // float4 rows (16-byte aligned: N a multiple of 4, cudaMalloc'd arrays)
    const dim3 grid((N + 127) / 128, (N + 7) / 8, N), block(32, 8);
    step_pair_xs<4><<<grid, block, 0, st>>>(c, ph, pl, qh, ql, oh, ol);
  } else if (N % 2 == 0) {
    const dim3 grid((N + 63) / 64, (N + 7) / 8, N), block(32, 8);
    step_pair_xs<2><<<grid, block, 0, st>>>(c, ph, pl, qh, ql, oh, ol);
  } else {
    const dim3 grid((N + 31) / 32, (N + 7) / 8, (N + PAIR_CZ - 1) / PAIR_CZ), block(32, 8);
    step_pair<<<grid, block, 0, st>>>(c, PAIR_CZ, ph, pl, qh, ql, oh, ol);
  }
  return cudaGetLastError();
}

cudaError_t launch_pair_from_ref(const double *ref, float *hi, float *lo, int N, cudaStream_t st) {
  const size_t V = (size_t)N * N * N;
  pair_from_ref<<<152 * 4, 256, 0, st>>>(ref, hi, lo, V, (size_t)N * N);
  return cudaGetLastError();
}

cudaError_t launch_pair_to_f64(const float *hi, const float *lo, double *out, int N, cudaStream_t st) {
  pair_to_f64<<<152 * 4, 256, 0, st>>>(hi, lo, out, (size_t)N * N * N);
  return cudaGetLastError();
}

}  // namespace phn
