// Island detection as connected-component labelling on the GPU.
//
// Replaces is_island + BFS + the seeding scan of Full_Analysis
// (islands.cpp:72-279, 778-840) for a first analysis (empty island history).
// Edges that are multiples of 32 (x) and 8 (y, z) take the tiled labelling:
//   1. ccl_tile: per 32 x 8 x 8 tile in shared memory, the mask, x-runs
//      linked by ballot and the -y/-z unions (union-find on tile-local
//      indices); every mask site links to its tile root, and the tile roots
//      are marked in a bit per site;
//   2. ccl_border_tiles: unions across tile faces only, each hooking the
//      larger root under the smaller by atomicCAS; a y or z union is skipped
//      where the -x sites of both ends are on the mask too (those two are
//      joined already, so are these);
//   3. ccl_resolve: each tile root's final root, root bits and counts.  Links
//      always point to smaller indices, so each root is the smallest site
//      index of its island;
// other edges link every site in global memory: ccl_init (mask, x-runs
// inside 32-site warp segments), ccl_merge (the unions, same skip rule),
// ccl_compress (parent = root, root bits), ccl_count_bits.  Then
//   4. ccl_number: islands numbered by their root in increasing index order,
//      which is the order in which the reference's linear scan seeds BFS, so
//      the labels equal the reference's b[] labels; tile roots take their
//      root's number (ccl_troot_ids), so ids[parent[i]] is the island of
//      every mask site;
//   5. statistics per island (size, energies, <phi>, peak): runs reduced in
//      the warp, merged per block in shared memory, then added to the FP64
//      per-island sums once per island per block (ccl_stats4, four sites per
//      lane; ccl_stats for edges that are not a multiple of 4); 6. records.
// Every loop terminates: a root search follows strictly decreasing indices,
// and a union retry strictly decreases the larger root.
#include <math.h>
#include <string.h>


#include <type_traits>

#include "ccl_math.h"
#include "phn_internal.h"
#include "site_terms.cuh"

namespace phn {

constexpr int CCL_THREADS = 256;

struct IslState {
  int *parent;     // [V]
  int *ids;        // [V] island id of each root (and, tiled, of each tile root)
  unsigned *tbits; // [W] tile roots, one bit per site (tiled labelling)
  unsigned *bits;  // [W] roots, one bit per site
  int *blk;        // [nblk] roots per block of CCL_THREADS words, then exclusive
                   // offsets; [ntile] the same per tile of SCAN_TILE blocks; [1] the total
  size_t W;        // 32-site words
  int nblk, ntile;
  // per-island arrays, grown on demand
  int cap;
  int *size;
  double *sums;                 // [cap][5]: pot, kin, grad, phi, (unused)
  unsigned long long *peak2;    // max peak_key per island
  long long *peakpos;           // reference index of the first max site
  double *peakval;
  int *seed;                    // root site (interior linear index)
  phn_island *rec;              // [cap] the records handed to the caller
};

// x, y, z of site i (i < 2^31)
__device__ __forceinline__ void site_xyz(const DivN &q, int N, size_t i, int &x, int &y, int &z) {
  const unsigned row = div_n(q, (unsigned)i), zz = div_n(q, row);
  x = (int)((unsigned)i - row * (unsigned)N);
  y = (int)(row - zz * (unsigned)N);
  z = (int)zz;
}

// Peak key of a site: the FP64 bits of phi^2 (non-negative, so the bits
// order like the values), or for plain FP32 fields the FP32 bits of |phi| --
// their squares are exact in FP64, so the two keys order the sites alike and
// tie alike.  ccl_stats takes the maximum key, ccl_peak the sites that hold it.
template <bool KAHAN, typename T>
__device__ __forceinline__ unsigned long long peak_key(const T *phi, const float *cphi, size_t i) {
  if constexpr (std::is_same<T, float>::value && !KAHAN) {
    return (unsigned long long)__float_as_uint(fabsf(phi[i]));
  } else {
    const double c = val_k<KAHAN>(phi, cphi, i);
    return (unsigned long long)__double_as_longlong(c * c);
  }
}

// Keys that order like the values for every sign (the peak of Delta).
__device__ __forceinline__ unsigned ordered_key(float v) {
  const unsigned u = __float_as_uint(v);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ unsigned long long ordered_key(double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// islands.cpp:76 in FP64; the FP32 form is the rare path of plain FP32 fields
// (a sum within 2^-19 of the threshold), kept out of line so that it is a
// branch and not issued for every site.
__device__ __forceinline__ bool ref_mask(double c, double p, double thr) {
  return __dadd_rn(__dmul_rn(__dmul_rn(c, c), 0.5), __dmul_rn(__dmul_rn(p, p), 0.5)) > thr;
}

__device__ __noinline__ bool ref_mask_f64(float c, float p, double thr) { return ref_mask(c, p, thr); }

// The island mask at site i = (x, y, z).
template <typename T, bool KAHAN>
__device__ __forceinline__ bool site_mask(const T *__restrict__ phi, const float *__restrict__ cphi,
                                          const T *__restrict__ pi, const float *__restrict__ cpi, int N, int mode,
                                          double thr, float thr_lo, float thr_hi, const Consts &k, size_t i, int x,
                                          int y, int z) {
  if (mode == PHN_ISLAND_REFERENCE) {
    // islands.cpp:76: Phi*Phi*0.5 + Pi*Pi*0.5 > thres*thres*0.5 (thr
    // holds the right side), in FP64.  Plain FP32 fields first try FP32
    // (ref_mask_f32, ccl_math.h); sums within the bracket, and NaN, take FP64.
    if constexpr (std::is_same<T, float>::value && !KAHAN) {
      const float cf = phi[i], pf = pi[i];
      const int d = ref_mask_f32(cf, pf, thr_lo, thr_hi);
      return d >= 0 ? d == 1 : ref_mask_f64(cf, pf, thr);
    } else {
      const double c = val_k<KAHAN>(phi, cphi, i), p = val_k<KAHAN>(pi, cpi, i);
      return ref_mask(c, p, thr);
    }
  }
  using A = typename std::conditional<std::is_same<T, float>::value, float, double>::type;
  if (mode == PHN_ISLAND_DELTA) return site_delta<A, KAHAN>(phi, cphi, pi, cpi, N, x, y, z, k) > (A)thr;
  return site_rho<A, KAHAN>(phi, cphi, pi, cpi, N, x, y, z, k) > (A)thr;
}

// The grid-stride loops below advance by whole warps of 32 consecutive
// sites (blocks are multiples of 32 threads), so site i is always handled by
// lane i % 32; ccl_merge relies on it to know which x links init made.
template <typename T, bool KAHAN>
__global__ void ccl_init(const T *__restrict__ phi, const float *__restrict__ cphi, const T *__restrict__ pi,
                         const float *__restrict__ cpi, int N, const DivN dn, int mode, double thr,
                         float thr_lo, float thr_hi, const Consts k, int *__restrict__ parent) {
  const size_t V = (size_t)N * N * N;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  for (size_t base = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) & ~(size_t)31; base < V;
       base += (size_t)gridDim.x * blockDim.x) {
    const size_t i = base + lane;
    bool m = false;
    int x = 0;
    if (i < V) {
      int y, z;
      site_xyz(dn, N, i, x, y, z);
      m = site_mask<T, KAHAN>(phi, cphi, pi, cpi, N, mode, thr, thr_lo, thr_hi, k, i, x, y, z);
    }
    // runs of mask sites along x within this segment: each site points at
    // the run's first site (a smaller index, as every link must)
    const unsigned mb = __ballot_sync(full, m);
    const unsigned joined = __ballot_sync(full, m && x != 0 && lane != 0 && ((mb >> (lane - 1)) & 1u));
    const unsigned heads = mb & ~joined;
    if (i < V) parent[i] = m ? (int)(base + (31 - __clz(heads & (full >> (31 - lane))))) : -1;
  }
}

// Union-find on site indices.  Every parent pointer points to a smaller or
// equal index; during the merge a root changes only by atomicCAS(root ->
// smaller root), and a non-root only by path halving, which stores one of its
// ancestors.  So concurrent finds may shorten each other's paths but never
// cut a link.  Halving is for the merge only: ccl_compress must leave every
// site pointing at its root, so it finds roots without writing (find_root_ro)
// -- a halving write there could replace a root just stored by another
// thread with an intermediate ancestor.
__device__ __forceinline__ int find_root_ro(const int *parent, int x) {
  int p = parent[x];
  while (p != x) {
    x = p;
    p = parent[x];
  }
  return x;
}

__device__ __forceinline__ int find_root(int *parent, int x) {
  int p = parent[x];
  while (p != x) {
    const int gp = parent[p];
    if (gp != p) parent[x] = gp;  // path halving: x now points two levels up
    x = p;
    p = gp;
  }
  return x;
}

__device__ void unite(int *parent, int a, int b) {
  while (true) {
    a = find_root(parent, a);
    b = find_root(parent, b);
    if (a == b) return;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    // hook the larger root under the smaller; retry if a stopped being a root
    if (atomicCAS(&parent[a], a, b) == a) return;
  }
}

__global__ void ccl_merge(int *__restrict__ parent, int N, const DivN dn, int zper) {
  const size_t V = (size_t)N * N * N, NN = (size_t)N * N;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < V; i += (size_t)gridDim.x * blockDim.x) {
    if (parent[i] < 0) continue;
    int x, y, z;
    site_xyz(dn, N, i, x, y, z);
    // -x: the periodic wrap, and the first lane of a segment (init links the rest)
    const bool left = x > 0 && parent[i - 1] >= 0;
    if (x == 0) {
      if (parent[i + N - 1] >= 0) unite(parent, (int)i, (int)(i + N - 1));
    } else if (left && (i & 31) == 0) {
      unite(parent, (int)i, (int)(i - 1));
    }
    // -y / -z: i-1 ~ i and j-1 ~ j along x, so with both -x sites on the mask
    // the pair (i-1, j-1) -- united, or skipped by the same rule further left
    // -- already joins i and j
    const size_t jy = (y == 0) ? i + (size_t)(N - 1) * N : i - N;
    if (parent[jy] >= 0 && !(left && parent[jy - 1] >= 0)) unite(parent, (int)i, (int)jy);
    if (z > 0 || zper) {
      const size_t jz = (z == 0) ? i + (size_t)(N - 1) * NN : i - NN;
      if (parent[jz] >= 0 && !(left && parent[jz - 1] >= 0)) unite(parent, (int)i, (int)jz);
    }
  }
}

// Tiled labelling for edges that are multiples of 32 (x) and 8 (y, z): a
// block labels a TILE_X x TILE_Y x TILE_Z tile in shared memory first (the
// same union-find on tile-local indices, whose order is the sites' index
// order, with the same skip rule), writes each mask site's link to the
// global index of its tile root, and ccl_border_tiles then unites across tile
// faces only: the -x union at lx = 0, -y at ly = 0, -z at lz = 0 (the skip
// rule needs the -x pair, which lies on the same face).  Shared-memory
// unions replace most global root searches.
constexpr int TILE_X = 32, TILE_Y = 8, TILE_Z = 8, TILE_SITES = TILE_X * TILE_Y * TILE_Z;

__device__ __forceinline__ int find_root_sh(volatile int *lp, int x) {
  int p = lp[x];
  while (p != x) {
    const int gp = lp[p];
    if (gp != p) lp[x] = gp;  // path halving, as find_root
    x = p;
    p = gp;
  }
  return x;
}

__device__ __forceinline__ int find_root_sh_ro(volatile int *lp, int x) {
  int p = lp[x];
  while (p != x) {
    x = p;
    p = lp[x];
  }
  return x;
}

__device__ __forceinline__ void unite_sh(int *lp, int a, int b) {
  while (true) {
    a = find_root_sh(lp, a);
    b = find_root_sh(lp, b);
    if (a == b) return;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    if (atomicCAS(&lp[a], a, b) == a) return;
  }
}

template <typename T, bool KAHAN>
__global__ void __launch_bounds__(TILE_X *TILE_Y) ccl_tile(const T *__restrict__ phi, const float *__restrict__ cphi,
                                                         const T *__restrict__ pi, const float *__restrict__ cpi,
                                                         int N, int mode, double thr, float thr_lo, float thr_hi,
                                                         const Consts k, int *__restrict__ parent,
                                                         unsigned *__restrict__ tbits) {
  static_assert(TILE_X == 32, "a tile row is one warp");
  __shared__ int lp[TILE_SITES];
  const int lx = threadIdx.x, ly = threadIdx.y;
  const int x0 = blockIdx.x * TILE_X, y0 = blockIdx.y * TILE_Y, z0 = blockIdx.z * TILE_Z;
  const int x = x0 + lx, y = y0 + ly;
  const size_t NN = (size_t)N * N;
  // the mask of the thread's TILE_Z sites, their loads issued together
  bool mk[TILE_Z];
  bool done = false;
  if constexpr (std::is_same<T, float>::value && !KAHAN) {
    if (mode == PHN_ISLAND_REFERENCE) {
      float cf[TILE_Z], pf[TILE_Z];
#pragma unroll
      for (int lz = 0; lz < TILE_Z; ++lz) {
        const size_t i = (size_t)(z0 + lz) * NN + (size_t)y * N + x;
        cf[lz] = phi[i];
        pf[lz] = pi[i];
      }
#pragma unroll
      for (int lz = 0; lz < TILE_Z; ++lz) {
        const int d = ref_mask_f32(cf[lz], pf[lz], thr_lo, thr_hi);
        mk[lz] = d >= 0 ? d == 1 : ref_mask_f64(cf[lz], pf[lz], thr);
      }
      done = true;
    }
  }
  if (!done) {
#pragma unroll
    for (int lz = 0; lz < TILE_Z; ++lz) {
      const size_t i = (size_t)(z0 + lz) * NN + (size_t)y * N + x;
      mk[lz] = site_mask<T, KAHAN>(phi, cphi, pi, cpi, N, mode, thr, thr_lo, thr_hi, k, i, x, y, z0 + lz);
    }
  }
  // a warp is one tile row: x-runs link to their first site by ballot, as
  // in ccl_init (the tile row starts the segment, so lx = 0 links nowhere);
  // the rows' mask words go to shared memory for the union rule
  __shared__ unsigned mrow[TILE_Z][TILE_Y];
  const unsigned full = 0xffffffffu;
  unsigned mbs[TILE_Z];
#pragma unroll
  for (int lz = 0; lz < TILE_Z; ++lz) {
    const int s = (lz * TILE_Y + ly) * TILE_X + lx;
    const unsigned mb = __ballot_sync(full, mk[lz]);
    const unsigned heads = mb & ~(mb << 1);
    mbs[lz] = mb;
    if (lx == 0) mrow[lz][ly] = mb;
    lp[s] = mk[lz] ? s - lx + (31 - __clz(heads & (full >> (31 - lx)))) : -1;
  }
  __syncthreads();
  // -y and -z unions by the skip rule, from the mask words: site s unites
  // with t when both are on the mask and not both of s-1, t-1 are
  // (b & ~(b << 1), b = the two rows' common mask).  A union joins the first
  // sites of the two x-runs (their links' targets), found from the words too.
  // Each warp first lists the unions of its eight rows (at most 16 per pair
  // of rows), then runs them with every lane busy: unions per row are few,
  // and a loop over the rows left most lanes idle in the root searches.
  __shared__ unsigned edges[TILE_Y][2 * TILE_Z * 16];
  {
    const unsigned le = full >> (31 - lx), lt = le >> 1;  // lanes 0..lx, 0..lx-1
    int ne = 0;                                           // uniform per warp
#pragma unroll
    for (int lz = 0; lz < TILE_Z; ++lz) {
      const unsigned me = mbs[lz];
      const unsigned wy = ly > 0 ? mrow[lz][ly - 1] : 0u, wz = lz > 0 ? mbs[lz - 1] : 0u;
      const unsigned by = me & wy, bz = me & wz;
      const unsigned uy = by & ~(by << 1), uz = bz & ~(bz << 1);
      const int row = (lz * TILE_Y + ly) * TILE_X;
      const unsigned hs = (unsigned)(row + 31 - __clz(me & ~(me << 1) & le));
      if ((uy >> lx) & 1u)
        edges[ly][ne + __popc(uy & lt)] = hs << 16 | (unsigned)(row - TILE_X + 31 - __clz(wy & ~(wy << 1) & le));
      ne += __popc(uy);
      if ((uz >> lx) & 1u)
        edges[ly][ne + __popc(uz & lt)] =
            hs << 16 | (unsigned)(row - TILE_X * TILE_Y + 31 - __clz(wz & ~(wz << 1) & le));
      ne += __popc(uz);
    }
    __syncwarp();
    for (int e = lx; e < ne; e += TILE_X) {
      const unsigned ab = edges[ly][e];
      unite_sh(lp, (int)(ab >> 16), (int)(ab & 0xffffu));
    }
  }
  __syncthreads();
  // each mask site links to its tile root's global index: the first site of
  // each x-run finds the root, the run's other sites take it by shuffle; the
  // tile roots' bits (one 32-bit word per tile row: N is a multiple of 32)
  // let the later passes visit the roots only
#pragma unroll
  for (int lz = 0; lz < TILE_Z; ++lz) {
    const int s = (lz * TILE_Y + ly) * TILE_X + lx;
    const size_t i = (size_t)(z0 + lz) * NN + (size_t)y * N + x;
    const unsigned mb = mbs[lz], heads = mb & ~(mb << 1);
    const bool m = (mb >> lx) & 1u;
    const int r0 = ((heads >> lx) & 1u) ? find_root_sh_ro(lp, s) : 0;
    const int r = __shfl_sync(full, r0, m ? 31 - __clz(heads & (full >> (31 - lx))) : lx);
    int g = -1;
    if (m) {
      const int rz = r / (TILE_X * TILE_Y), ry = (r / TILE_X) % TILE_Y, rx = r % TILE_X;
      g = (int)((size_t)(z0 + rz) * NN + (size_t)(y0 + ry) * N + (x0 + rx));
    }
    parent[i] = g;
    const unsigned tb = __ballot_sync(full, m && r == s);
    if (lx == 0) tbits[i >> 5] = tb;
  }
}

// Unions across tile faces (see ccl_tile), one block per tile: warp w takes
// the -y face's row at lz = w and the -z face's row at ly = w, threads
// 0-63 the -x face's column.  parent[] of a mask site is a tile root (or an
// ancestor of one, after a path-halving write), and every union hooks one
// tile root under another, so after this pass the tile roots alone carry
// the cross-tile structure.

// Whether the face pair (i, j) needs a union: both on the mask, and not
// dropped by the skip rule of ccl_merge (with i-1 and j-1 on the mask too,
// the pair (i-1, j-1) -- united here or skipped by the same rule -- joins i
// and j).
__device__ __forceinline__ bool face_pair(const int *parent, size_t i, size_t j, bool skip_rule) {
  if (parent[i] < 0 || parent[j] < 0) return false;
  return !(skip_rule && parent[i - 1] >= 0 && parent[j - 1] >= 0);
}

__global__ void __launch_bounds__(CCL_THREADS) ccl_border_tiles(int *__restrict__ parent, int N, int zper) {
  static_assert(CCL_THREADS == TILE_X * TILE_Y && TILE_Y == TILE_Z, "one row of each face per warp");
  // each warp lists its faces' unions, then runs them with every lane busy
  // (a face row holds a few; the root searches are global-memory latency)
  __shared__ int2 pairs[CCL_THREADS / 32][3 * 32];
  const unsigned full = 0xffffffffu;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int x0 = blockIdx.x * TILE_X, y0 = blockIdx.y * TILE_Y, z0 = blockIdx.z * TILE_Z;
  const size_t NN = (size_t)N * N;
  const int x = x0 + lane;
  const unsigned lt = (1u << lane) - 1u;
  int np = 0;  // uniform per warp
  auto offer = [&](bool want, size_t i, size_t j) {
    const unsigned b = __ballot_sync(full, want);
    if (want) pairs[w][np + __popc(b & lt)] = make_int2((int)i, (int)j);
    np += __popc(b);
  };
  {  // -y face, periodic
    const size_t i = (size_t)(z0 + w) * NN + (size_t)y0 * N + x;
    const size_t j = y0 == 0 ? i + (size_t)(N - 1) * N : i - N;
    offer(face_pair(parent, i, j, x > 0), i, j);
  }
  if (z0 > 0 || zper) {  // -z face, open on one rank unless asked periodic (uniform per block)
    const size_t i = (size_t)z0 * NN + (size_t)(y0 + w) * N + x;
    const size_t j = z0 == 0 ? i + (size_t)(N - 1) * NN : i - NN;
    offer(face_pair(parent, i, j, x > 0), i, j);
  }
  if (w < TILE_Y * TILE_Z / 32) {  // -x face, periodic (warps 0 and 1)
    const size_t i = (size_t)(z0 + t / TILE_Y) * NN + (size_t)(y0 + t % TILE_Y) * N + x0;
    const size_t j = x0 == 0 ? i + N - 1 : i - 1;
    offer(face_pair(parent, i, j, false), i, j);
  }
  __syncwarp();
  for (int e = lane; e < np; e += 32) unite(parent, pairs[w][e].x, pairs[w][e].y);
}

// Roots per block of CCL_THREADS threads, into blk[blockIdx.x].
__device__ __forceinline__ void block_count(int c, int *blk) {
  __shared__ int cnt[CCL_THREADS / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
  if ((threadIdx.x & 31) == 0) cnt[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < CCL_THREADS / 32; ++w) s += cnt[w];
    blk[blockIdx.x] = s;
  }
}

// Tiled labelling: every tile root's final root.  One thread per 32-site
// word of the tile-root bits; a tile root that is not a root gets its root
// written (root searches of other threads still end at the same root), a
// root sets its bit in bits[].  Counts the roots per block of CCL_THREADS
// words for the numbering scan.
__global__ void __launch_bounds__(CCL_THREADS) ccl_resolve(int *__restrict__ parent, const unsigned *__restrict__ tbits,
                                                          size_t W, unsigned *__restrict__ bits, int *__restrict__ blk) {
  const size_t w = blockIdx.x * (size_t)CCL_THREADS + threadIdx.x;
  unsigned rb = 0;
  if (w < W) {
    for (unsigned b = tbits[w]; b; b &= b - 1u) {
      const int kb = __ffs(b) - 1;
      const int tr = (int)(w * 32 + kb);
      const int r = find_root_ro(parent, tr);
      if (r == tr) rb |= 1u << kb;
      else parent[tr] = r;
    }
    bits[w] = rb;
  }
  block_count(__popc(rb), blk);
}

// Untiled labelling: parent[i] = root(i) for every mask site, and the roots'
// bits (a warp covers one aligned 32-site word).
__global__ void __launch_bounds__(CCL_THREADS) ccl_compress(int *__restrict__ parent, size_t V,
                                                           unsigned *__restrict__ bits) {
  const size_t i = blockIdx.x * (size_t)CCL_THREADS + threadIdx.x;
  bool root = false;
  if (i < V) {
    const int p = parent[i];
    if (p >= 0) {
      const int r = find_root_ro(parent, (int)i);
      parent[i] = r;
      root = (r == (int)i);
    }
  }
  const unsigned b = __ballot_sync(0xffffffffu, root);
  if ((threadIdx.x & 31) == 0 && i < V) bits[i >> 5] = b;
}

// roots per block of CCL_THREADS words (untiled labelling)
__global__ void __launch_bounds__(CCL_THREADS) ccl_count_bits(const unsigned *__restrict__ bits, size_t W,
                                                             int *__restrict__ blk) {
  const size_t w = blockIdx.x * (size_t)CCL_THREADS + threadIdx.x;
  block_count(w < W ? __popc(bits[w]) : 0, blk);
}

// Exclusive scan of the block counts in two levels: each block of
// ccl_scan_tiles scans SCAN_TILE consecutive counts in place (coalesced) and
// writes the tile's total; ccl_scan then scans the tile totals in one block.
// ccl_number adds both offsets.
constexpr int SCAN_TILE = 1024;

__global__ void __launch_bounds__(SCAN_TILE) ccl_scan_tiles(int *__restrict__ blk, int n, int *__restrict__ tile) {
  __shared__ int wsum[SCAN_TILE / 32];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const size_t b = (size_t)blockIdx.x * SCAN_TILE + t;
  const int v = b < (size_t)n ? blk[b] : 0;
  int s = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, s, off);
    if (lane >= off) s += u;
  }
  if (lane == 31) wsum[warp] = s;
  __syncthreads();
  if (warp == 0) {
    int w = wsum[lane];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += u;
    }
    wsum[lane] = w;  // inclusive totals of warps 0..lane
  }
  __syncthreads();
  const int ex = s - v + (warp ? wsum[warp - 1] : 0);
  if (b < (size_t)n) blk[b] = ex;
  if (t == SCAN_TILE - 1) tile[blockIdx.x] = wsum[SCAN_TILE / 32 - 1];
}

// exclusive scan of the tile totals, one block, fixed order
__global__ void ccl_scan(int *__restrict__ blk, int n, int *__restrict__ total) {
  __shared__ int part[1024];
  const int t = threadIdx.x;
  const int per = (n + 1023) / 1024;
  const int b0 = t * per, b1 = min(n, b0 + per);
  int s = 0;
  for (int b = b0; b < b1; ++b) s += blk[b];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    int run = 0;
    for (int j = 0; j < 1024; ++j) {
      const int v = part[j];
      part[j] = run;
      run += v;
    }
    *total = run;
  }
  __syncthreads();
  int run = part[t];
  for (int b = b0; b < b1; ++b) {
    const int v = blk[b];
    blk[b] = run;
    run += v;
  }
}

// Islands are numbered by their root in increasing site order: the rank of
// each root bit, from the scanned block counts and a scan of the popcounts
// inside the block.
__global__ void __launch_bounds__(CCL_THREADS) ccl_number(const unsigned *__restrict__ bits, size_t W,
                                                         const int *__restrict__ blk, const int *__restrict__ tile,
                                                         int *__restrict__ ids, int *__restrict__ seed, int cap) {
  __shared__ int wsum[CCL_THREADS / 32];
  const size_t w = blockIdx.x * (size_t)CCL_THREADS + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned b = w < W ? bits[w] : 0u;
  const int c = __popc(b);
  int incl = c;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += u;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  int off = blk[blockIdx.x] + tile[blockIdx.x / SCAN_TILE] + incl - c;
  for (int v = 0; v < warp; ++v) off += wsum[v];
  for (; b; b &= b - 1u) {
    const int r = (int)(w * 32 + (__ffs(b) - 1));
    ids[r] = off;
    if (off < cap) seed[off] = r;
    ++off;
  }
}

// Tiled labelling: each tile root that is not a root takes its root's
// island number, so that ids[parent[i]] is the island of every mask site.
__global__ void __launch_bounds__(CCL_THREADS) ccl_troot_ids(const unsigned *__restrict__ tbits, size_t W,
                                                            const int *__restrict__ parent, int *__restrict__ ids) {
  const size_t w = blockIdx.x * (size_t)CCL_THREADS + threadIdx.x;
  if (w >= W) return;
  for (unsigned b = tbits[w]; b; b &= b - 1u) {
    const int tr = (int)(w * 32 + (__ffs(b) - 1));
    const int r = parent[tr];
    if (r != tr) ids[tr] = ids[r];
  }
}

// Per-island sums.  Block b owns the STATS_SITES consecutive sites
// [b STATS_SITES, (b+1) STATS_SITES) (whole x rows); a warp takes 32
// consecutive sites at a time.  Sites of one island along a row form runs,
// which a segmented inclusive scan over the lanes reduces (size, PotEn, KinEn,
// GradEn and phi sums, max phi^2); each run's last lane merges its sums into
// the block's shared-memory table keyed by island id, and the block adds each
// table entry to the global sums once.  An island that spans the lattice (a
// percolating mask) so costs one global atomic per block, not one per site:
// same-address atomics from every warp were what bounded this pass.  A run
// that finds the table full adds to the global sums directly.
constexpr int STATS_SITES = 8192;
constexpr int STATS_SLOTS = 512;  // power of two; with the run scratch under 48 KB of static shared memory

// One island's sums in a block's table: pot, kin, grad, phi.  FP64 fields
// add in FP64.  FP32 fields keep each sum as a float pair hi + lo without any
// FP64 instruction: atomicAdd(hi, v) returns the old value, atom.add.f32
// rounds to nearest even, so the error of that addition is the TwoSum term
// (old + v) - RN(old + v) (Knuth, TAOCP vol. 2, 4.2.2), which goes into lo.
// The pair tracks the exact sum but for lo's own (second-order) rounding.
template <typename A>
struct StatsSlot {
  double s[4];
  unsigned long long peak2;
  int size, id;
  __device__ void clear() { s[0] = s[1] = s[2] = s[3] = 0.0; }
  __device__ void add(int j, double v) { atomicAdd(&s[j], v); }
  __device__ double sum(int j) const { return s[j]; }
};

template <>
struct StatsSlot<float> {
  float hi[4], lo[4];
  unsigned long long peak2;
  int size, id;
  __device__ void clear() {
    for (int j = 0; j < 4; ++j) hi[j] = lo[j] = 0.f;
  }
  __device__ void add(int j, float v) {
    const float old = atomicAdd(&hi[j], v);
    const float s = __fadd_rn(old, v), bb = __fsub_rn(s, old);
    const float err = __fadd_rn(__fsub_rn(old, __fsub_rn(s, bb)), __fsub_rn(v, bb));
    if (err != 0.f) atomicAdd(&lo[j], err);
  }
  __device__ double sum(int j) const { return (double)hi[j] + (double)lo[j]; }
};

template <typename A>
struct alignas(16) RunSums {  // 16-byte aligned: the scratch copies move as vectors
  A pot, kin, grad, cs;
  unsigned long long pk;
  int n;
};

template <typename A>
__device__ __forceinline__ void stats_global(int id, int n, A pot, A kin, A grad, A cs, unsigned long long pk,
                                             int *size, double *sums, unsigned long long *peak2) {
  atomicAdd(&size[id], n);
  atomicAdd(&sums[(size_t)id * 4 + 0], (double)pot);
  atomicAdd(&sums[(size_t)id * 4 + 1], (double)kin);
  atomicAdd(&sums[(size_t)id * 4 + 2], (double)grad);
  atomicAdd(&sums[(size_t)id * 4 + 3], (double)cs);
  atomicMax(&peak2[id], pk);
}

// One run's sums into the block's table: open addressing on the island id,
// linear probing; a full table sends the run to the global sums.
template <typename A>
__device__ __forceinline__ void table_update(StatsSlot<A> *table, int id, const RunSums<A> &r, int *size,
                                             double *sums, unsigned long long *peak2) {
  unsigned h = ((unsigned)id * 2654435761u) & (STATS_SLOTS - 1);
  int slot = -1;
  for (int probe = 0; probe < STATS_SLOTS; ++probe) {
    const int old = atomicCAS(&table[h].id, -1, id);
    if (old == -1 || old == id) {
      slot = (int)h;
      break;
    }
    h = (h + 1) & (STATS_SLOTS - 1);
  }
  if (slot >= 0) {
    atomicAdd(&table[slot].size, r.n);
    table[slot].add(0, r.pot);
    table[slot].add(1, r.kin);
    table[slot].add(2, r.grad);
    table[slot].add(3, r.cs);
    atomicMax(&table[slot].peak2, r.pk);
  } else {
    stats_global(id, r.n, r.pot, r.kin, r.grad, r.cs, r.pk, size, sums, peak2);
  }
}

template <typename A>
__device__ __forceinline__ void table_clear(StatsSlot<A> *table) {
  for (int j = threadIdx.x; j < STATS_SLOTS; j += CCL_THREADS) {
    table[j].clear();
    table[j].peak2 = 0;
    table[j].size = 0;
    table[j].id = -1;
  }
}

template <typename A>
__device__ __forceinline__ void table_flush(const StatsSlot<A> *table, int *size, double *sums,
                                            unsigned long long *peak2) {
  for (int j = threadIdx.x; j < STATS_SLOTS; j += CCL_THREADS) {
    const StatsSlot<A> &t = table[j];
    if (t.id >= 0) stats_global(t.id, t.size, t.sum(0), t.sum(1), t.sum(2), t.sum(3), t.peak2, size, sums, peak2);
  }
}

// The statistics for any edge, one site per lane (edges that are not a
// multiple of 4).
template <typename T, bool KAHAN>
__global__ void __launch_bounds__(CCL_THREADS) ccl_stats(const T *__restrict__ phi, const float *__restrict__ cphi,
                                                        const T *__restrict__ pi, const float *__restrict__ cpi,
                                                        const int *__restrict__ parent, const int *__restrict__ ids,
                                                        int N, const DivN dn, const Consts k, int dpeak,
                                                        int *__restrict__ size,
                                                        double *__restrict__ sums,
                                                        unsigned long long *__restrict__ peak2) {
  // FP32 fields: per-site terms and the in-warp scan in FP32 (GB300's FP64
  // rate would otherwise bound the pass); FP64 fields: FP64.  The global
  // per-island sums are FP64 either way.
  using A = typename std::conditional<std::is_same<T, float>::value, float, double>::type;
  __shared__ StatsSlot<A> table[STATS_SLOTS];
  __shared__ RunSums<A> scratch[CCL_THREADS / 32][32];
  table_clear(table);
  __syncthreads();
  const size_t V = (size_t)N * N * N, NN = (size_t)N * N;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t s0 = (size_t)blockIdx.x * STATS_SITES;
  const size_t s1 = s0 + STATS_SITES < V ? s0 + STATS_SITES : V;
  // chunk loop: uniform per warp, so every lane takes part in the collectives
  for (size_t base = s0 + (size_t)warp * 32; base < s1; base += (size_t)(CCL_THREADS / 32) * 32) {
    const size_t i = base + lane;
    int id = -1, n = 0;
    A pot = 0, kin = 0, grad = 0, cs = 0;
    unsigned long long pk = 0;
    const int r = i < s1 ? parent[i] : -1;
    if (__ballot_sync(full, r >= 0) == 0) continue;  // uniform per warp
    if (r >= 0) {
      id = ids[r];
      int x, y, z;
      site_xyz(dn, N, i, x, y, z);
      const A c = val_as<A, KAHAN>(phi, cphi, i), p = val_as<A, KAHAN>(pi, cpi, i);
      const A fx = val_as<A, KAHAN>(phi, cphi, i - x + (x + 1 == N ? 0 : x + 1));
      const A fy = val_as<A, KAHAN>(phi, cphi, (size_t)z * NN + (size_t)(y + 1 == N ? 0 : y + 1) * N + x);
      const A fz = val_as<A, KAHAN>(phi, cphi, (size_t)(z + 1 == N ? 0 : z + 1) * NN + (size_t)y * N + x);
      // BFS accumulators (islands.cpp:131-198)
      grad = grad_half(c, fx, fy, fz, inv_a2_of<A>(k));
      kin = site_kinetic(k, c, p);
      pot = site_potential(k, c, c * c);
      cs = c;
      n = 1;
      pk = dpeak ? ordered_key((double)delta_of<A>(kin, grad, pot)) : peak_key<KAHAN>(phi, cphi, i);
    }
    const int prev = __shfl_up_sync(full, id, 1);
    const unsigned heads = __ballot_sync(full, lane == 0 || prev != id);
    const int start = 31 - __clz(heads & (full >> (31 - lane)));  // first lane of my run
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const A up = __shfl_up_sync(full, pot, off), uk = __shfl_up_sync(full, kin, off);
      const A ug = __shfl_up_sync(full, grad, off), uc = __shfl_up_sync(full, cs, off);
      const int un = __shfl_up_sync(full, n, off);
      const unsigned long long upk = __shfl_up_sync(full, pk, off);
      if (lane - off >= start) {
        pot += up;
        kin += uk;
        grad += ug;
        cs += uc;
        n += un;
        pk = upk > pk ? upk : pk;
      }
    }
    const int next = __shfl_down_sync(full, id, 1);
    const bool end = (lane == 31 || next != id) && id >= 0;
    // The runs of one island in this chunk (a cluster winding through it)
    // combine first, in lane order, so that the table takes one update per
    // island per chunk: updates of one slot serialise, and the FP64 ones on
    // GB300's narrow FP64 pipe.
    const unsigned grp = __match_any_sync(full, end ? id : -1 - lane);
    if (end) scratch[warp][lane] = RunSums<A>{pot, kin, grad, cs, pk, n};
    __syncwarp();
    if (end && (grp & ((1u << lane) - 1u)) == 0) {
      for (unsigned b = grp & (grp - 1u); b; b &= b - 1u) {
        const RunSums<A> &o = scratch[warp][__ffs(b) - 1];
        pot += o.pot;
        kin += o.kin;
        grad += o.grad;
        cs += o.cs;
        n += o.n;
        pk = o.pk > pk ? o.pk : pk;
      }
      table_update(table, id, RunSums<A>{pot, kin, grad, cs, pk, n}, size, sums, peak2);
    }
    __syncwarp();  // scratch is rewritten by the next chunk
  }
  __syncthreads();
  table_flush(table, size, sums, peak2);
}

// ---------------------------------------------------------------------------
// The statistics with four consecutive x-sites per lane (edges that are a
// multiple of 4): a warp covers 128 sites, so the warp collectives -- the
// segmented scan, the grouping of runs by island, the table updates -- run
// once per 128 sites instead of once per 32, and every field is read as
// 16-byte vectors.
//
// Mask sites adjacent along x in one row belong to one island, so the runs
// are found from the mask alone and the island number is looked up once per
// run.  A lane splits its four sites at their gaps: L, the run through its
// first site; R, the run through its last; M, a run between two gaps (at most
// one in four sites).  A lane whose four sites are all on the mask passes L
// on.  The carry C (the run through the lane's last site, summed over the
// lanes it spans) is a segmented inclusive scan over the lanes; a segment
// starts at every lane that does not continue the previous lane's run (its
// first site off the mask, the previous lane's last site off it, or a new
// row).  Closed runs: L plus the previous lane's carry, at a lane with a gap;
// M; and C where the next lane does not continue it.
//
// Plain FP32 fields pack the peak as (|phi| bits, ~index): the maximum is
// the largest |phi| and, among equal ones, the smallest index, which is the
// peak position itself -- no second pass over the sites.
template <typename A>
__device__ __forceinline__ void run_zero(RunSums<A> &r) {
  r.pot = r.kin = r.grad = r.cs = (A)0;
  r.pk = 0;
  r.n = 0;
}

template <typename A>
__device__ __forceinline__ void run_add(RunSums<A> &r, const RunSums<A> &o) {
  r.pot += o.pot;
  r.kin += o.kin;
  r.grad += o.grad;
  r.cs += o.cs;
  r.n += o.n;
  r.pk = o.pk > r.pk ? o.pk : r.pk;
}

template <typename A>
__device__ __forceinline__ RunSums<A> run_shfl_up(const RunSums<A> &r, int off) {
  const unsigned full = 0xffffffffu;
  return RunSums<A>{__shfl_up_sync(full, r.pot, off), __shfl_up_sync(full, r.kin, off),
                    __shfl_up_sync(full, r.grad, off), __shfl_up_sync(full, r.cs, off),
                    __shfl_up_sync(full, r.pk, off),  __shfl_up_sync(full, r.n, off)};
}

template <typename A>
__device__ __forceinline__ RunSums<A> run_shfl_down(const RunSums<A> &r, int off) {
  const unsigned full = 0xffffffffu;
  return RunSums<A>{__shfl_down_sync(full, r.pot, off), __shfl_down_sync(full, r.kin, off),
                    __shfl_down_sync(full, r.grad, off), __shfl_down_sync(full, r.cs, off),
                    __shfl_down_sync(full, r.pk, off),  __shfl_down_sync(full, r.n, off)};
}

// One round of table updates: the lanes with u set offer (id, r); the offers
// of one island combine first, so that the table takes one update per island
// per round.  When every offer is of one island (runs of the spanning
// cluster, most often) they combine by a shuffle tree over the lanes from the
// first to the last offer, the others in lane order through the scratch row.
template <typename A>
__device__ __forceinline__ void table_round(bool u, int id, RunSums<A> r, StatsSlot<A> *table, RunSums<A> *scratch,
                                            int lane, int *size, double *sums, unsigned long long *peak2) {
  const unsigned full = 0xffffffffu;
  const unsigned um = __ballot_sync(full, u);
  if (um == 0u) return;
  const int first = __ffs(um) - 1, last = 31 - __clz(um);
  const int id0 = __shfl_sync(full, id, first);
  if (__all_sync(full, !u || id == id0)) {
    if (!u) run_zero(r);
    for (int off = 1; first + off <= last; off <<= 1) {  // uniform per warp
      const RunSums<A> o = run_shfl_down(r, off);
      if (((lane - first) & (2 * off - 1)) == 0 && lane + off <= last) run_add(r, o);
    }
    if (lane == first) table_update(table, id0, r, size, sums, peak2);
    return;
  }
  const unsigned grp = __match_any_sync(full, u ? id : -1 - lane);
  if (u) scratch[lane] = r;
  __syncwarp();
  if (u && (grp & ((1u << lane) - 1u)) == 0) {
    for (unsigned b = grp & (grp - 1u); b; b &= b - 1u) run_add(r, scratch[__ffs(b) - 1]);
    table_update(table, id, r, size, sums, peak2);
  }
  __syncwarp();  // scratch is rewritten by the next round
}

// Four consecutive values of a field in arithmetic A (16-byte loads; i0 is a
// multiple of 4).
template <typename A, bool KAHAN, typename T>
__device__ __forceinline__ void load4(const T *__restrict__ f, const float *__restrict__ comp, size_t i0, A v[4]) {
  if constexpr (std::is_same<T, double>::value) {
    const double2 a = *(const double2 *)(f + i0), b = *(const double2 *)(f + i0 + 2);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
  } else {
    const float4 a = *(const float4 *)(f + i0);
    if constexpr (KAHAN) {
      const float4 c = *(const float4 *)(comp + i0);
      v[0] = (A)((double)a.x - (double)c.x);
      v[1] = (A)((double)a.y - (double)c.y);
      v[2] = (A)((double)a.z - (double)c.z);
      v[3] = (A)((double)a.w - (double)c.w);
    } else {
      v[0] = a.x;
      v[1] = a.y;
      v[2] = a.z;
      v[3] = a.w;
    }
  }
}

template <typename T, bool KAHAN>
__global__ void __launch_bounds__(CCL_THREADS) ccl_stats4(const T *__restrict__ phi, const float *__restrict__ cphi,
                                                         const T *__restrict__ pi, const float *__restrict__ cpi,
                                                         const int *__restrict__ parent, const int *__restrict__ ids,
                                                         int N, const DivN dn, const Consts k, int dpeak,
                                                         int *__restrict__ size, double *__restrict__ sums,
                                                         unsigned long long *__restrict__ peak2) {
  using A = typename std::conditional<std::is_same<T, float>::value, float, double>::type;
  constexpr bool PACKED = std::is_same<T, float>::value && !KAHAN;
  constexpr int WARP_SITES = 32 * 4;
  __shared__ StatsSlot<A> table[STATS_SLOTS];
  __shared__ RunSums<A> scratch[CCL_THREADS / 32][32];
  table_clear(table);
  __syncthreads();
  const size_t V = (size_t)N * N * N, NN = (size_t)N * N;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t s0 = (size_t)blockIdx.x * STATS_SITES;
  const size_t s1 = s0 + STATS_SITES < V ? s0 + STATS_SITES : V;
  // chunk loop: uniform per warp, so every lane takes part in the collectives
  for (size_t base = s0 + (size_t)warp * WARP_SITES; base < s1; base += (size_t)(CCL_THREADS / 32) * WARP_SITES) {
    const size_t i0 = base + 4 * (size_t)lane;  // V is a multiple of 4: all four sites or none
    int4 pr = make_int4(-1, -1, -1, -1);
    if (i0 < s1) pr = *(const int4 *)(parent + i0);
    const int prv[4] = {pr.x, pr.y, pr.z, pr.w};
    const bool any = pr.x >= 0 || pr.y >= 0 || pr.z >= 0 || pr.w >= 0;
    if (__ballot_sync(full, any) == 0) continue;  // uniform per warp
    // the island numbers of the four sites, fetched with the fields (a run
    // that closes in this lane takes its number from one of its sites)
    int idv[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) idv[j] = prv[j] >= 0 ? ids[prv[j]] : -1;
    int x0 = 0, y = 0, z = 0;
    if (i0 < s1) site_xyz(dn, N, i0, x0, y, z);
    RunSums<A> L, M, R;
    run_zero(L);
    run_zero(M);
    run_zero(R);
    int mid = -1, rid = -1;  // the island of M and of R
    if (any) {
      A c[4], p[4], fy[4], fz[4];
      const size_t row = (size_t)z * NN + (size_t)y * N;
      load4<A, KAHAN>(phi, cphi, i0, c);
      load4<A, KAHAN>(pi, cpi, i0, p);
      load4<A, KAHAN>(phi, cphi, (size_t)z * NN + (size_t)(y + 1 == N ? 0 : y + 1) * N + x0, fy);
      load4<A, KAHAN>(phi, cphi, (size_t)(z + 1 == N ? 0 : z + 1) * NN + (size_t)y * N + x0, fz);
      const A fx3 = val_as<A, KAHAN>(phi, cphi, row + (x0 + 4 == N ? 0 : x0 + 4));
      bool gap = false;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (prv[j] < 0) {
          if (gap && R.n > 0) {
            M = R;
            mid = rid;
          }
          run_zero(R);
          gap = true;
        } else {
          const A cj = c[j], fx = j < 3 ? c[j + 1] : fx3;
          RunSums<A> t;
          // BFS accumulators (islands.cpp:131-198)
          t.grad = grad_half(cj, fx, fy[j], fz[j], inv_a2_of<A>(k));
          t.kin = site_kinetic(k, cj, p[j]);
          t.pot = site_potential(k, cj, cj * cj);
          t.cs = cj;
          t.n = 1;
          if constexpr (PACKED) {
            const unsigned key = dpeak ? ordered_key(delta_of<A>(t.kin, t.grad, t.pot)) : __float_as_uint(fabsf(cj));
            t.pk = ((unsigned long long)key << 32) | (unsigned long long)(0xffffffffu - (unsigned)(i0 + j));
          } else {
            t.pk = dpeak ? ordered_key((double)delta_of<A>(t.kin, t.grad, t.pot)) : peak_key<KAHAN>(phi, cphi, i0 + j);
          }
          if (!gap) {
            run_add(L, t);
          } else {
            run_add(R, t);
            rid = idv[j];
          }
        }
      }
    }
    const bool m0 = pr.x >= 0, m3 = pr.w >= 0;
    const bool through = pr.x >= 0 && pr.y >= 0 && pr.z >= 0 && pr.w >= 0;
    const bool m3prev = __shfl_up_sync(full, m3, 1);
    const bool conn = lane > 0 && m0 && m3prev && x0 != 0;
    // segmented inclusive scan of the carries; it stops at the first step
    // that no lane's segment reaches back to (the longest segment sets the
    // number of steps)
    RunSums<A> C = through ? L : R;
    const unsigned heads = __ballot_sync(full, !(through && conn));
    const int start = 31 - __clz(heads & (full >> (31 - lane)));
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      if (!__any_sync(full, lane - off >= start)) break;  // uniform per warp
      const RunSums<A> u = run_shfl_up(C, off);
      if (lane - off >= start) run_add(C, u);
    }
    const bool conn_next = __shfl_down_sync(full, conn, 1);
    bool u1 = C.n > 0 && (lane == 31 || !conn_next);  // the carry closes here
    bool u2 = !through && m0;                        // L closes at the lane's first gap
    bool u3 = M.n > 0;
    if (__any_sync(full, u2 && conn)) {
      const RunSums<A> Cp = run_shfl_up(C, 1);
      if (u2 && conn) run_add(L, Cp);
    }
    const int id1 = u1 ? idv[3] : -1, id2 = u2 ? idv[0] : -1, id3 = u3 ? mid : -1;
    // a lane's own closed runs of one island combine first
    if (u3 && u2 && id3 == id2) {
      run_add(L, M);
      u3 = false;
    }
    if (u1 && u2 && id1 == id2) {
      run_add(L, C);
      u1 = false;
    }
    if (u1 && u3 && id1 == id3) {
      run_add(M, C);
      u1 = false;
    }
    // the lane's closed runs in order (L, M, C, whichever close here): the
    // first round takes every lane's first, so the later rounds are short or
    // skipped
    const bool w1 = (u2 && u3) || (u1 && (u2 || u3)), w2 = u2 && u3 && u1;
    table_round(u2 || u3 || u1, u2 ? id2 : (u3 ? id3 : id1), u2 ? L : (u3 ? M : C), table, scratch[warp], lane, size,
                sums, peak2);
    table_round(w1, (u2 && u3) ? id3 : id1, (u2 && u3) ? M : C, table, scratch[warp], lane, size, sums, peak2);
    table_round(w2, id1, C, table, scratch[warp], lane, size, sums, peak2);
  }
  __syncthreads();
  table_flush(table, size, sums, peak2);
}

// Plain FP32 fields: the peak position from the packed key (ccl_stats4).
__global__ void ccl_peak_unpack(const unsigned long long *__restrict__ peak2, int n, long long NN,
                                long long *__restrict__ peakpos) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    peakpos[j] = (long long)(0xffffffffu - (unsigned)(peak2[j] & 0xffffffffull)) + NN;
}

// Delta of site i from the BFS summands, as the statistics kernels form it.
template <typename T, bool KAHAN>
__device__ __forceinline__ double site_delta_stats(const T *phi, const float *cphi, const T *pi, const float *cpi,
                                                   int N, const DivN &dn, const Consts &k, size_t i) {
  using A = typename std::conditional<std::is_same<T, float>::value, float, double>::type;
  int x, y, z;
  site_xyz(dn, N, i, x, y, z);
  const size_t NN = (size_t)N * N;
  const A c = val_as<A, KAHAN>(phi, cphi, i), p = val_as<A, KAHAN>(pi, cpi, i);
  const A fx = val_as<A, KAHAN>(phi, cphi, i - x + (x + 1 == N ? 0 : x + 1));
  const A fy = val_as<A, KAHAN>(phi, cphi, (size_t)z * NN + (size_t)(y + 1 == N ? 0 : y + 1) * N + x);
  const A fz = val_as<A, KAHAN>(phi, cphi, (size_t)(z + 1 == N ? 0 : z + 1) * NN + (size_t)y * N + x);
  return (double)delta_of<A>(site_kinetic(k, c, p), grad_half(c, fx, fy, fz, inv_a2_of<A>(k)),
                             site_potential(k, c, c * c));
}

// The sites that hold each island's peak key; dpeak: the key of Delta.
template <typename T, bool KAHAN>
__global__ void ccl_peak(const T *__restrict__ phi, const float *__restrict__ cphi, const T *__restrict__ pi,
                         const float *__restrict__ cpi, const int *__restrict__ parent, const int *__restrict__ ids,
                         int N, const DivN dn, const Consts k, int dpeak,
                         const unsigned long long *__restrict__ peak2, long long *__restrict__ peakpos) {
  const size_t V = (size_t)N * N * N, NN = (size_t)N * N;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < V; i += (size_t)gridDim.x * blockDim.x) {
    const int r = parent[i];
    if (r < 0) continue;
    const int id = ids[r];
    const unsigned long long key =
        dpeak ? ordered_key(site_delta_stats<T, KAHAN>(phi, cphi, pi, cpi, N, dn, k, i)) : peak_key<KAHAN>(phi, cphi, i);
    if (key == peak2[id]) atomicMin(&peakpos[id], (long long)(i + NN));  // reference index (Nc = 1)
  }
}

// Peak_value: phi at the peak (islands.cpp:256-258), or Delta there (:259-260).
template <typename T, bool KAHAN>
__global__ void ccl_peakval(const T *__restrict__ phi, const float *__restrict__ cphi, const T *__restrict__ pi,
                            const float *__restrict__ cpi, int N, const DivN dn, const Consts k, int dpeak, int n,
                            const long long *__restrict__ peakpos, double *__restrict__ peakval) {
  const size_t NN = (size_t)N * N, V = NN * N;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    // every island has a site, so its peak lies on the lattice; a position
    // off it (an island whose statistics were never written) reads nothing
    const size_t i = (size_t)peakpos[j] - NN;
    if (i >= V) {
      peakval[j] = __longlong_as_double(0x7ff8000000000000ll);
      continue;
    }
    peakval[j] = dpeak ? site_delta_stats<T, KAHAN>(phi, cphi, pi, cpi, N, dn, k, i) : val(phi, cphi, i);
  }
}

// labels in the reference layout: ghost slabs -1, interior island ids
__global__ void ccl_labels(const int *__restrict__ parent, const int *__restrict__ ids, int N, int *__restrict__ out) {
  const size_t NN = (size_t)N * N, V = NN * N, total = NN * (N + 2);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int v = -1;
    if (i >= NN && i < NN + V) {
      const int r = parent[i - NN];
      if (r >= 0) v = ids[r];
    }
    out[i] = v;
  }
}

// Island of each queried site (reference-layout index; -1 outside the mask or
// the interior).
__global__ void ccl_lookup(const int *__restrict__ parent, const int *__restrict__ ids, int N,
                           const long long *__restrict__ pos, int n, int *__restrict__ out) {
  const size_t NN = (size_t)N * N, V = NN * N;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const long long k = pos[j];
    int v = -1;
    if (k >= (long long)NN && k < (long long)(NN + V)) {
      const int r = parent[k - NN];
      if (r >= 0) v = ids[r];
    }
    out[j] = v;
  }
}

// Labels in the reference layout through a map from island number to label.
__global__ void ccl_labels_mapped(const int *__restrict__ parent, const int *__restrict__ ids,
                                  const int *__restrict__ map, int N, int *__restrict__ out) {
  const size_t NN = (size_t)N * N, V = NN * N, total = NN * (N + 2);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int v = -1;
    if (i >= NN && i < NN + V) {
      const int r = parent[i - NN];
      if (r >= 0) v = map[ids[r]];
    }
    out[i] = v;
  }
}

// The caller's records (islands.cpp:239-262 units), assembled on the device
// so that one copy returns them.  volume = ((size a) a) a and the energies
// sum * a^3 as the reference's cV factors; no operation here can contract.
__global__ void ccl_records(const int *__restrict__ size, const double *__restrict__ sums,
                            const long long *__restrict__ peakpos, const double *__restrict__ peakval,
                            const int *__restrict__ seed, int n, double a, double cell, long long NN,
                            phn_island *__restrict__ out) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    phn_island I;
    const double sz = (double)size[j];
    I.index = (double)j;
    I.size = sz;
    I.volume = __dmul_rn(__dmul_rn(__dmul_rn(sz, a), a), a);  // cV = NN*a_t*a_t*a_eta (islands.cpp:241)
    I.pot_en = __dmul_rn(sums[(size_t)j * 4 + 0], cell);
    I.kin_en = __dmul_rn(sums[(size_t)j * 4 + 1], cell);
    I.grad_en = __dmul_rn(sums[(size_t)j * 4 + 2], cell);
    I.av_phi = __ddiv_rn(sums[(size_t)j * 4 + 3], sz);
    I.peak_pos = (double)peakpos[j];
    I.peak_value = peakval[j];
    I.seed_pos = (double)((long long)seed[j] + NN);
    out[j] = I;
  }
}

__global__ void fill_ll(long long *p, long long v, int n) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) p[j] = v;
}

static void free_isl_arrays(IslState *s) {
  cudaFree(s->size);
  cudaFree(s->sums);
  cudaFree(s->peak2);
  cudaFree(s->peakpos);
  cudaFree(s->peakval);
  cudaFree(s->seed);
  cudaFree(s->rec);
  s->rec = nullptr;
  s->size = nullptr;
  s->sums = nullptr;
  s->peak2 = nullptr;
  s->peakpos = nullptr;
  s->peakval = nullptr;
  s->seed = nullptr;
  s->cap = 0;
}

void islands_release(phn_handle *h) {
  IslState *s = (IslState *)h->isl;
  if (!s) return;
  cudaFree(s->parent);
  cudaFree(s->ids);
  cudaFree(s->tbits);
  cudaFree(s->bits);
  cudaFree(s->blk);
  free_isl_arrays(s);
  delete s;
  h->isl = nullptr;
}

static int grid_blocks(size_t n) {
  size_t b = (n + CCL_THREADS - 1) / CCL_THREADS;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b ? b : 1);
}

template <typename T>
static int run_islands(phn_handle *h, const T *phi, const T *pi, double thres, int mode, int zper, int *labels,
                       phn_island *out, int max_out, int *n_islands, const phn_island **d_out = nullptr) {
  const int N = h->p.N;
  const size_t V = h->V;
  cudaStream_t st = h->stream;
  const float *cphi = h->p.precision == PHN_FP32_KAHAN ? h->cphi : nullptr;
  const float *cpi = h->p.precision == PHN_FP32_KAHAN ? h->cpi : nullptr;
  if (!h->isl) {
    IslState *s = new IslState();
    memset(s, 0, sizeof(*s));
    h->isl = s;
    s->W = (V + 31) / 32;
    s->nblk = (int)((s->W + CCL_THREADS - 1) / CCL_THREADS);
    s->ntile = (s->nblk + SCAN_TILE - 1) / SCAN_TILE;
    cudaError_t e = cudaMalloc(&s->parent, V * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&s->ids, V * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&s->tbits, s->W * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&s->bits, s->W * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&s->blk, ((size_t)s->nblk + s->ntile + 1) * sizeof(int));
    if (e != cudaSuccess) {
      islands_release(h);
      return cuda_error(e, "island buffers");
    }
  }
  IslState *s = (IslState *)h->isl;
  const double thr = mode == PHN_ISLAND_REFERENCE ? (thres * thres * 0.5) : thres;
  const int gb = grid_blocks(V);
  const Consts k = consts_now(h);
  const DivN dn = make_divn((unsigned)N);
  float thr_lo, thr_hi;  // the FP32 bracket of the reference mask (site_mask)
  mask_bracket(thr, &thr_lo, &thr_hi);
  const bool tiled = N % TILE_X == 0 && N % TILE_Y == 0 && N % TILE_Z == 0;
  if (tiled) {
    // tile labels, face unions, then the tile roots' roots and the root bits
    const dim3 tg(N / TILE_X, N / TILE_Y, N / TILE_Z), tb(TILE_X, TILE_Y);
    if (cphi)
      ccl_tile<T, true><<<tg, tb, 0, st>>>(phi, cphi, pi, cpi, N, mode, thr, thr_lo, thr_hi, k, s->parent, s->tbits);
    else
      ccl_tile<T, false><<<tg, tb, 0, st>>>(phi, cphi, pi, cpi, N, mode, thr, thr_lo, thr_hi, k, s->parent, s->tbits);
    ccl_border_tiles<<<tg, CCL_THREADS, 0, st>>>(s->parent, N, zper);
    ccl_resolve<<<s->nblk, CCL_THREADS, 0, st>>>(s->parent, s->tbits, s->W, s->bits, s->blk);
  } else {
    if (cphi)
      ccl_init<T, true><<<gb, CCL_THREADS, 0, st>>>(phi, cphi, pi, cpi, N, dn, mode, thr, thr_lo, thr_hi, k,
                                                   s->parent);
    else
      ccl_init<T, false><<<gb, CCL_THREADS, 0, st>>>(phi, cphi, pi, cpi, N, dn, mode, thr, thr_lo, thr_hi, k,
                                                    s->parent);
    ccl_merge<<<gb, CCL_THREADS, 0, st>>>(s->parent, N, dn, zper);
    ccl_compress<<<(unsigned)((V + CCL_THREADS - 1) / CCL_THREADS), CCL_THREADS, 0, st>>>(s->parent, V, s->bits);
    ccl_count_bits<<<s->nblk, CCL_THREADS, 0, st>>>(s->bits, s->W, s->blk);
  }
  int *tile = s->blk + s->nblk;
  ccl_scan_tiles<<<s->ntile, SCAN_TILE, 0, st>>>(s->blk, s->nblk, tile);
  ccl_scan<<<1, 1024, 0, st>>>(tile, s->ntile, tile + s->ntile);
  h->launches += tiled ? 5 : 6;
  int count = 0;
  cudaError_t e = cudaMemcpyAsync(&count, tile + s->ntile, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "island count");
  if (count > s->cap) {
    free_isl_arrays(s);
    const int cap = count + count / 4 + 64;
    e = cudaMalloc(&s->size, cap * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&s->sums, (size_t)cap * 4 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->peak2, cap * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&s->peakpos, cap * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&s->peakval, cap * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->seed, cap * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&s->rec, cap * sizeof(phn_island));
    if (e != cudaSuccess) {
      free_isl_arrays(s);
      return cuda_error(e, "island arrays");
    }
    s->cap = cap;
  }
  ccl_number<<<s->nblk, CCL_THREADS, 0, st>>>(s->bits, s->W, s->blk, tile, s->ids, s->seed, s->cap);
  h->launches++;
  if (tiled) {
    ccl_troot_ids<<<s->nblk, CCL_THREADS, 0, st>>>(s->tbits, s->W, s->parent, s->ids);
    h->launches++;
  }
  if (count > 0) {
    // four sites per lane where rows hold whole groups of four; plain FP32
    // fields then take the peak from the packed key, the others in a
    // second pass over the sites
    const bool x4 = N % 4 == 0;
    const bool packed = x4 && std::is_same<T, float>::value && !cphi;
    cudaMemsetAsync(s->size, 0, count * sizeof(int), st);
    cudaMemsetAsync(s->sums, 0, (size_t)count * 4 * sizeof(double), st);
    cudaMemsetAsync(s->peak2, 0, count * sizeof(unsigned long long), st);
    if (!packed) {
      fill_ll<<<(count + 255) / 256, 256, 0, st>>>(s->peakpos, LLONG_MAX, count);
      h->launches++;
    }
    const unsigned sb = (unsigned)((V + STATS_SITES - 1) / STATS_SITES);
    const int dpeak = mode == PHN_ISLAND_DELTA;
    if (x4) {
      if (cphi)
        ccl_stats4<T, true><<<sb, CCL_THREADS, 0, st>>>(phi, cphi, pi, cpi, s->parent, s->ids, N, dn, k, dpeak,
                                                        s->size, s->sums, s->peak2);
      else
        ccl_stats4<T, false><<<sb, CCL_THREADS, 0, st>>>(phi, cphi, pi, cpi, s->parent, s->ids, N, dn, k, dpeak,
                                                         s->size, s->sums, s->peak2);
    } else {
      if (cphi)
        ccl_stats<T, true><<<sb, CCL_THREADS, 0, st>>>(phi, cphi, pi, cpi, s->parent, s->ids, N, dn, k, dpeak,
                                                       s->size, s->sums, s->peak2);
      else
        ccl_stats<T, false><<<sb, CCL_THREADS, 0, st>>>(phi, cphi, pi, cpi, s->parent, s->ids, N, dn, k, dpeak,
                                                        s->size, s->sums, s->peak2);
    }
    if (packed) {
      ccl_peak_unpack<<<(count + 255) / 256, 256, 0, st>>>(s->peak2, count, (long long)N * N, s->peakpos);
    } else if (cphi) {
      ccl_peak<T, true><<<gb, CCL_THREADS, 0, st>>>(phi, cphi, pi, cpi, s->parent, s->ids, N, dn, k, dpeak, s->peak2,
                                                    s->peakpos);
    } else {
      ccl_peak<T, false><<<gb, CCL_THREADS, 0, st>>>(phi, cphi, pi, cpi, s->parent, s->ids, N, dn, k, dpeak, s->peak2,
                                                     s->peakpos);
    }
    if (cphi)
      ccl_peakval<T, true><<<(count + 255) / 256, 256, 0, st>>>(phi, cphi, pi, cpi, N, dn, k, dpeak, count,
                                                                s->peakpos, s->peakval);
    else
      ccl_peakval<T, false><<<(count + 255) / 256, 256, 0, st>>>(phi, cphi, pi, cpi, N, dn, k, dpeak, count,
                                                                 s->peakpos, s->peakval);
    h->launches += 3;
  }
  if (labels) {
    const size_t total = (size_t)N * N * (N + 2);
    int *d_lab = nullptr;
    e = cudaMallocAsync((void **)&d_lab, total * sizeof(int), st);
    if (e != cudaSuccess) return cuda_error(e, "label buffer");
    ccl_labels<<<grid_blocks(total), CCL_THREADS, 0, st>>>(s->parent, s->ids, N, d_lab);
    h->launches++;
    e = cudaMemcpyAsync(labels, d_lab, total * sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d_lab, st);
    if (e != cudaSuccess) return cuda_error(e, "label readback");
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "island kernels");
  if (d_out) {  // every record, left in the handle's device buffer
    *d_out = nullptr;
    if (count > 0) {
      const double a = h->p.a, cell = (a * a) * a;
      ccl_records<<<(count + 255) / 256, 256, 0, st>>>(s->size, s->sums, s->peakpos, s->peakval, s->seed, count, a,
                                                       cell, (long long)N * N, s->rec);
      h->launches++;
      e = cudaGetLastError();
      if (e != cudaSuccess) return cuda_error(e, "island records");
      *d_out = s->rec;
    }
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "islands");
    if (n_islands) *n_islands = count;
    return PHN_OK;
  }
  const int n_out = count < max_out ? count : max_out;
  if (out && n_out > 0) {
    const double a = h->p.a, cell = (a * a) * a;
    ccl_records<<<(n_out + 255) / 256, 256, 0, st>>>(s->size, s->sums, s->peakpos, s->peakval, s->seed, n_out, a,
                                                     cell, (long long)N * N, s->rec);
    h->launches++;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, s->rec, (size_t)n_out * sizeof(phn_island), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "island readback");
  } else {
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "islands");
  }
  if (n_islands) *n_islands = count;
  if (out && count > max_out) return set_error(PHN_ERR_TRUNCATED, "%d islands, %d records written", count, max_out);
  return PHN_OK;
}

}  // namespace phn

using namespace phn;

// Labels of the last phn_islands call mapped through map[island] (n entries),
// into host memory (reference layout).
int phn::islands_labels_mapped(phn_handle *h, const int *map, int n, int *labels) {
  IslState *s = (IslState *)h->isl;
  if (!s) return set_error(PHN_ERR_INVALID, "no island labelling on this handle yet");
  cudaStream_t st = h->stream;
  const int N = h->p.N;
  const size_t total = (size_t)N * N * (N + 2);
  int *d_map = nullptr, *d_lab = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&d_map, (size_t)(n > 0 ? n : 1) * sizeof(int), st);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_lab, total * sizeof(int), st);
  if (e == cudaSuccess && n > 0) e = cudaMemcpyAsync(d_map, map, n * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    ccl_labels_mapped<<<grid_blocks(total), CCL_THREADS, 0, st>>>(s->parent, s->ids, d_map, N, d_lab);
    h->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(labels, d_lab, total * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d_map, st);
  cudaFreeAsync(d_lab, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? PHN_OK : cuda_error(e, "mapped labels");
}

extern "C" int phn_islands_lookup(phn_handle *h, const long long *pos, int n, int *island) {
  if (!h || (n > 0 && (!pos || !island)) || n < 0) return set_error(PHN_ERR_INVALID, "bad argument");
  IslState *s = (IslState *)h->isl;
  if (!s) return set_error(PHN_ERR_INVALID, "phn_islands first");
  if (n == 0) return PHN_OK;
  cudaStream_t st = h->stream;
  long long *d_pos = nullptr;
  int *d_out = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&d_pos, n * sizeof(long long), st);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_out, n * sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_pos, pos, n * sizeof(long long), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    ccl_lookup<<<(n + 255) / 256, 256, 0, st>>>(s->parent, s->ids, h->p.N, d_pos, n, d_out);
    h->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(island, d_out, n * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d_pos, st);
  cudaFreeAsync(d_out, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? PHN_OK : cuda_error(e, "island lookup");
}

extern "C" int phn_islands(phn_handle *h, double thres, int mode, int z_periodic, int *labels, phn_island *out,
                           int max_out, int *n_islands) {
  if (!h) return set_error(PHN_ERR_INVALID, "handle is NULL");
  if (h->p.Nc != 1) return set_error(PHN_ERR_UNSUPPORTED, "islands need Nc == 1");
  if (mode != PHN_ISLAND_REFERENCE && mode != PHN_ISLAND_ENERGY && mode != PHN_ISLAND_DELTA)
    return set_error(PHN_ERR_INVALID, "mode %d", mode);
  if (mode == PHN_ISLAND_DELTA && h->p.potential < 2)
    return set_error(PHN_ERR_UNSUPPORTED, "the Delta mask has no form for theory %d (the reference's withEnergyPS "
                     "build compiles for theories 2-5)", h->p.potential);
  if (h->V > (size_t)0x7fffffff) return set_error(PHN_ERR_UNSUPPORTED, "lattice too large for 32-bit labels");
  if (max_out < 0) return set_error(PHN_ERR_INVALID, "max_out < 0");
  if (h->p.precision == PHN_FP64)
    return run_islands<double>(h, (const double *)h->phi[h->cur], (const double *)h->pi, thres, mode, z_periodic,
                               labels, out, max_out, n_islands);
  return run_islands<float>(h, (const float *)h->phi[h->cur], (const float *)h->pi, thres, mode, z_periodic, labels,
                            out, max_out, n_islands);
}

extern "C" int phn_islands_device(phn_handle *h, double thres, int mode, int z_periodic,
                                  const phn_island **d_records, int *n_islands) {
  if (!h || !d_records || !n_islands) return set_error(PHN_ERR_INVALID, "bad argument");
  if (h->p.Nc != 1) return set_error(PHN_ERR_UNSUPPORTED, "islands need Nc == 1");
  if (mode != PHN_ISLAND_REFERENCE && mode != PHN_ISLAND_ENERGY && mode != PHN_ISLAND_DELTA)
    return set_error(PHN_ERR_INVALID, "mode %d", mode);
  if (mode == PHN_ISLAND_DELTA && h->p.potential < 2)
    return set_error(PHN_ERR_UNSUPPORTED, "the Delta mask has no form for theory %d", h->p.potential);
  if (h->V > (size_t)0x7fffffff) return set_error(PHN_ERR_UNSUPPORTED, "lattice too large for 32-bit labels");
  if (h->p.precision == PHN_FP64)
    return run_islands<double>(h, (const double *)h->phi[h->cur], (const double *)h->pi, thres, mode, z_periodic,
                               nullptr, nullptr, 0, n_islands, d_records);
  return run_islands<float>(h, (const float *)h->phi[h->cur], (const float *)h->pi, thres, mode, z_periodic,
                            nullptr, nullptr, 0, n_islands, d_records);
}
