// Leapfrog in FP32 pairs: double-float arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2
// (about 48 significant bits).  Additions use Knuth's TwoSum for the high
// words and add the low words into the error (the "sloppy" double-float sum),
// products use the FMA error of the high words (Dekker's product with an
// FMA, T. J. Dekker, Numer. Math. 18, 1971; Knuth, TAOCP vol. 2, 4.2.2), and
// every result is renormalised with Fast2Sum.  GB300's FP64 rate is a small
// fraction of its FP32 rate; a pair step costs about 130 FP32 operations per
// site and reaches FP64-class accuracy (a 32^3 phi^6 run of 1000 steps stays
// within 2e-9 of FP64, against 5e-7 for plain FP32).
//
// It serves the adjoint's forward solve: the sigmoid objective amplifies a
// change of the final state some 400-fold into the gradient, and compensated
// FP32 does not help there, because the increments dt F and dt pi are
// themselves rounded to FP32 every step (an error correlated from step to
// step, which grows linearly).  Here force, increments and updates are all
// pair arithmetic.  Theories 0 and 1, Nc = 1, static box.
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
  const F2 l = f2_mul(c, c);
  F2 coef = k.c4;
  if (k.theory == 0) coef = f2_madd(k.c4, l, k.c6);
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
// phi keeps its sign between them, and their sum is accumulated with TwoSum;
// the low words' differences add plainly (they are ~2^-24 of the high
// words').  A 32^3 phi^6 run of 1000 steps stays as close to FP64 as with
// full pair differences (1.5e-9), at a third of the Laplacian's cost.
__device__ __forceinline__ F2 pair_force_w(const PairConsts &k, F2 c, const F2 nb[6]) {
  float acc = 0.f, err = 0.f, lo = 0.f;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const float d = __fsub_rn(nb[j].hi, c.hi);
    const float t = __fadd_rn(acc, d);
    const float bb = __fsub_rn(t, acc);
    err = __fadd_rn(err, __fadd_rn(__fsub_rn(acc, __fsub_rn(t, bb)), __fsub_rn(d, bb)));
    acc = t;
    lo = __fadd_rn(lo, __fsub_rn(nb[j].lo, c.lo));
  }
  const F2 s = f2_fast(acc, __fadd_rn(err, lo));
  return pair_potential_force(k, c, s);
}

// Four consecutive x-sites per thread, one plane: pi += fk F(phi) in place,
// phi' = phi + fd pi'.  Both words of phi and pi move as float4; the x
// neighbours outside the four come as scalars.  N a multiple of 4.
__global__ void __launch_bounds__(256, 4) step_pair_x4(const PairConsts k, const float *__restrict__ ph,
                                                    const float *__restrict__ pl, float *__restrict__ qh,
                                                    float *__restrict__ ql, float *__restrict__ oh,
                                                    float *__restrict__ ol) {
  const int N = k.N;
  const int x0 = 4 * (blockIdx.x * 32 + threadIdx.x), y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
  if (x0 >= N || y >= N) return;
  const size_t NN = (size_t)N * N;
  const size_t plane = (size_t)z * NN, row = plane + (size_t)y * N;
  const size_t i = row + x0;
  const size_t iyp = plane + (size_t)(y + 1 == N ? 0 : y + 1) * N + x0;
  const size_t iym = plane + (size_t)(y == 0 ? N - 1 : y - 1) * N + x0;
  const size_t izp = (size_t)(z + 1 == N ? 0 : z + 1) * NN + (size_t)y * N + x0;
  const size_t izm = (size_t)(z == 0 ? N - 1 : z - 1) * NN + (size_t)y * N + x0;
  const size_t ixl = row + (x0 == 0 ? N - 1 : x0 - 1), ixr = row + (x0 + 4 == N ? 0 : x0 + 4);
  const float4 ch = *(const float4 *)(ph + i), cl = *(const float4 *)(pl + i);
  const float4 yph = *(const float4 *)(ph + iyp), ypl = *(const float4 *)(pl + iyp);
  const float4 ymh = *(const float4 *)(ph + iym), yml = *(const float4 *)(pl + iym);
  const float4 zph = *(const float4 *)(ph + izp), zpl = *(const float4 *)(pl + izp);
  const float4 zmh = *(const float4 *)(ph + izm), zml = *(const float4 *)(pl + izm);
  const F2 xl = F2{ph[ixl], pl[ixl]}, xr = F2{ph[ixr], pl[ixr]};
  const float4 pqh = *(const float4 *)(qh + i), pql = *(const float4 *)(ql + i);
  const float chv[4] = {ch.x, ch.y, ch.z, ch.w}, clv[4] = {cl.x, cl.y, cl.z, cl.w};
  const float yphv[4] = {yph.x, yph.y, yph.z, yph.w}, yplv[4] = {ypl.x, ypl.y, ypl.z, ypl.w};
  const float ymhv[4] = {ymh.x, ymh.y, ymh.z, ymh.w}, ymlv[4] = {yml.x, yml.y, yml.z, yml.w};
  const float zphv[4] = {zph.x, zph.y, zph.z, zph.w}, zplv[4] = {zpl.x, zpl.y, zpl.z, zpl.w};
  const float zmhv[4] = {zmh.x, zmh.y, zmh.z, zmh.w}, zmlv[4] = {zml.x, zml.y, zml.z, zml.w};
  const float qhv[4] = {pqh.x, pqh.y, pqh.z, pqh.w}, qlv[4] = {pql.x, pql.y, pql.z, pql.w};
  float nqh[4], nql[4], nph[4], npl[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const F2 c = F2{chv[j], clv[j]};
    const F2 left = j == 0 ? xl : F2{chv[j - 1], clv[j - 1]};
    const F2 right = j == 3 ? xr : F2{chv[j + 1], clv[j + 1]};
    const F2 nb[6] = {right, left, F2{yphv[j], yplv[j]}, F2{ymhv[j], ymlv[j]}, F2{zphv[j], zplv[j]},
                      F2{zmhv[j], zmlv[j]}};
    const F2 f = pair_force_w(k, c, nb);
    const F2 q = f2_madd(F2{qhv[j], qlv[j]}, f, k.fk);
    const F2 p = f2_madd(c, q, k.fd);
    nqh[j] = q.hi;
    nql[j] = q.lo;
    nph[j] = p.hi;
    npl[j] = p.lo;
  }
  *(float4 *)(qh + i) = make_float4(nqh[0], nqh[1], nqh[2], nqh[3]);
  *(float4 *)(ql + i) = make_float4(nql[0], nql[1], nql[2], nql[3]);
  *(float4 *)(oh + i) = make_float4(nph[0], nph[1], nph[2], nph[3]);
  *(float4 *)(ol + i) = make_float4(npl[0], npl[1], npl[2], npl[3]);
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
    const F2 p = f2_madd(c, q, k.fd);
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
  c.c6 = f2_of(k.theory == 0 ? 1.0 / (k.kappa * k.kappa * k.c120) : 0.0);
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
  if (N % 4 == 0) {  // float4 rows (16-byte aligned: N a multiple of 4, cudaMalloc'd arrays)
    const dim3 grid((N + 127) / 128, (N + 7) / 8, N), block(32, 8);
    step_pair_x4<<<grid, block, 0, st>>>(c, ph, pl, qh, ql, oh, ol);
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
