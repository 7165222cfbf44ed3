// gd_pipeline.cu -- the exact-DBSCAN kernels for one instance.
//
// Replaces, in the reference (CUDA-DClust+):
//   host bbox + bin widths        main.cu:166-207           -> k_bbox_partial, k_params
//   INDEXING_STRUCTURE/insertData indexing.cu:54-118        -> k_keys (cell keys)
//   thrust::sort_by_key           main.cu:332               -> gdprim::radix_sort_pairs
//   INDEXING_ADJUSTMENT           indexing.cu:23-51         -> k_run_flags/k_run_scatter/
//                                                              k_cell_counts + scan (cell table)
//   DBSCAN kernel + searchPoints  dbscan.cu:254-474         -> k_core (core flags)
//   MarkAsCandidate + host merge  dbscan.cu:189-222, 25-187 -> k_union (device union-find)
//   GetDbscanResult               dbscan.cu:225-251         -> k_roots, k_label, k_border,
//                                                              k_scatter_labels
//
// Grid: fine cells of side f = eps * m, m = 0.5 * (1 + 2^-16) by default, keyed
// x-major.  Two points of one cell are always neighbours (cell diagonal
// <= 0.87 eps), and every neighbour of a point lies within +-2 cells per axis.
// A cell holding >= minpts points is therefore all core ("dense") without a
// single distance evaluation, and all core points of a cell are in one cluster.
//
// Precision modes (template flag F32):
//   F32 = false: every pair decision is the float64 predicate (gd_internal.cuh).
//   F32 = true : the pair is first measured in float32 on bbox-centred
//                coordinates; only pairs whose float32 d2 falls inside a proven
//                rounding band around eps^2 are re-tested with the float64
//                predicate.  Outside the band the float32 decision provably
//                equals the float64 one, so labels stay bit-exact.
#include <cfloat>
#include <climits>

#include "gd_internal.cuh"
#include "gd_launch.h"

namespace gd {

// ------------------------------------------------------------------ bbox
constexpr int kBboxThreads = 256;

// Doubles ordered as int64 (monotone for non-NaN values): min/max run on the
// integer pipe instead of the much slower float64 pipe of this GPU.
__device__ __forceinline__ long long ord_of(double v) {
  long long b = __double_as_longlong(v);
  return b >= 0 ? b : b ^ 0x7fffffffffffffffLL;
}
__device__ __forceinline__ double dbl_of(long long o) {
  return __longlong_as_double(o >= 0 ? o : o ^ 0x7fffffffffffffffLL);
}

template <int D>
__global__ void __launch_bounds__(kBboxThreads)
k_bbox_partial(const double* __restrict__ pts, int64_t n, long long* __restrict__ partial,
               int* __restrict__ flags) {
  long long lo[D], hi[D];
#pragma unroll
  for (int k = 0; k < D; ++k) { lo[k] = LLONG_MAX; hi[k] = LLONG_MIN; }
  bool bad = false;
  const long long* __restrict__ bits = reinterpret_cast<const long long*>(pts);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      long long bv = bits[i * D + k];
      bad |= (bv & 0x7ff0000000000000LL) == 0x7ff0000000000000LL;
      long long o = bv >= 0 ? bv : bv ^ 0x7fffffffffffffffLL;
      lo[k] = min(lo[k], o);
      hi[k] = max(hi[k], o);
    }
  }
  __shared__ long long s[2 * D][kBboxThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < D; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = min(lo[k], __shfl_xor_sync(kFull, lo[k], o));
      hi[k] = max(hi[k], __shfl_xor_sync(kFull, hi[k], o));
    }
    if (lane == 0) { s[k][w] = lo[k]; s[D + k][w] = hi[k]; }
  }
  if (__any_sync(kFull, bad) && lane == 0) atomicOr(flags, kFlagNonFinite);
  __syncthreads();
  if (threadIdx.x < 2 * D) {
    const int k = threadIdx.x;
    long long v = s[k][0];
    for (int j = 1; j < kBboxThreads / 32; ++j) v = k < D ? min(v, s[k][j]) : max(v, s[k][j]);
    partial[blockIdx.x * 2 * D + k] = v;
  }
}

// One block: reduce the partial boxes; thread 0 derives the grid and the
// float32 band.
template <int D>
__global__ void __launch_bounds__(256)
k_params(const long long* __restrict__ partial, int nblocks, DevParams* P, double eps, int minpts,
         double cell_mult, uint64_t max_cells, const int* __restrict__ flags) {
  __shared__ long long s[2 * D][256];
  long long lo[D], hi[D];
#pragma unroll
  for (int k = 0; k < D; ++k) { lo[k] = LLONG_MAX; hi[k] = LLONG_MIN; }
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < D; ++k) {
      lo[k] = min(lo[k], partial[b * 2 * D + k]);
      hi[k] = max(hi[k], partial[b * 2 * D + k + D]);
    }
#pragma unroll
  for (int k = 0; k < D; ++k) { s[k][threadIdx.x] = lo[k]; s[D + k][threadIdx.x] = hi[k]; }
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st)
#pragma unroll
      for (int k = 0; k < D; ++k) {
        s[k][threadIdx.x] = min(s[k][threadIdx.x], s[k][threadIdx.x + st]);
        s[D + k][threadIdx.x] = max(s[D + k][threadIdx.x], s[D + k][threadIdx.x + st]);
      }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  DevParams p;
  int fl = *flags;
  for (int k = 0; k < 3; ++k) { p.lo[k] = 0; p.hi[k] = 0; p.centre[k] = 0; p.G[k] = 1; }
  for (int k = 0; k < D; ++k) {
    p.lo[k] = dbl_of(s[k][0]);
    p.hi[k] = dbl_of(s[D + k][0]);
    p.centre[k] = 0.5 * p.lo[k] + 0.5 * p.hi[k];
  }
  p.dim = D;
  p.minpts = minpts;
  p.eps = eps;
  p.eps2 = __dmul_rn(eps, eps);
  p.f = __dmul_rn(eps, cell_mult);
  p.inv_f = 1.0 / p.f;
  double cells = 1.0;
  uint64_t C = 1;
  for (int k = 0; k < D; ++k) {
    double t = floor(__dmul_rn(__dsub_rn(p.hi[k], p.lo[k]), p.inv_f)) + 1.0;
    if (!(t < 2147483648.0)) { fl |= kFlagGridTooLarge; t = 1.0; }
    p.G[k] = (int64_t)t;
    cells *= t;
    C *= (uint64_t)p.G[k];
  }
  // keys must fit 62 bits; a grid beyond the dense-table limit uses the hash
  if (!(cells < 4.0e18)) fl |= kFlagGridTooLarge;
  p.sparse = (cells > (double)max_cells || C > max_cells) ? 1 : 0;
  p.C = C;
  int bits = 0;
  while (bits < 63 && (C - 1) >> bits) ++bits;
  p.key_bits = bits;
  // box-test shortcut and float32 filter need every |x| <= eps * 2^30
  double maxabs = 0, R = 0;
  for (int k = 0; k < D; ++k) {
    maxabs = fmax(maxabs, fmax(fabs(p.lo[k]), fabs(p.hi[k])));
    R = fmax(R, fmax(p.hi[k] - p.centre[k], p.centre[k] - p.lo[k]));
  }
  if (maxabs <= eps * 1073741824.0) {
    p.eps2_in = __dmul_rn(p.eps2, 1.0 - 1.0 / 524288.0);    // 1 - 2^-19
  } else {
    p.eps2_in = -1.0;
    fl |= kFlagNoShortcut;
  }
  // float32 band.  a_k = fl32(x_k - c_k) is off from x_k - c_k by at most
  // ea = R 2^-24 (R bounds |x_k - c_k|).  For a pair with true squared distance
  // S, the float32 value s = fl(fl(u0^2) + ...), u_k = fl32(a_pk - a_qk), obeys
  //   |s - S| <= (S + 4 ea sqrt(D S) + 4 D ea^2)(D + 3) 2^-24
  //              + 4 ea sqrt(D S) + 4 D ea^2  =: B(S)
  // (coordinate error, one rounding per subtraction, D roundings in the FMA
  // chain).  Evaluated at S = 2 eps^2 and padded by 1.5 this is bmax.  Then
  //   s < L = eps^2 (1 - 2^-17) - bmax  =>  S < eps^2 (1 - 2^-17)
  //        =>  float64 d2 <= eps2_in  =>  neighbour both ways (box test passes);
  //   s > H = eps^2 (1 + 2^-17) + bmax  =>  float64 d2 > eps2  =>  not a neighbour.
  // L is rounded down and H up to float32.  Pairs with L <= s <= H take the
  // float64 predicate.  The filter is off (fp64 only) when the bound is not small.
  {
    const double u32 = 1.0 / 16777216.0;               // 2^-24
    R = R * (1.0 + 1e-12) + 1e-300;
    const double ea = R * u32 * (1.0 + 1e-8);          // |fl32(x - c) - (x - c)|
    const double e2 = p.eps2;
    const double rs = sqrt(2.0 * e2) * sqrt((double)D);
    double bmax = (2.0 * e2 + 4.0 * ea * rs + 4.0 * D * ea * ea) * (D + 3) * u32
                  + 4.0 * ea * rs + 4.0 * D * ea * ea;
    bmax *= 1.5;
    const double L = e2 * (1.0 - 1.0 / 131072.0) - bmax;   // 2^-17
    const double H = e2 * (1.0 + 1.0 / 131072.0) + bmax;
    const bool ok = !(fl & kFlagNoShortcut) && e2 > 1e-30 && R < 1e30 && L > 0.25 * e2 &&
                    H < 4.0 * e2;
    p.eps2_lo32 = ok ? __double2float_rd(L) : -1.0f;
    p.eps2_hi32 = ok ? __double2float_ru(H) : -1.0f;
    // Cell-level classification.  A point's position inside its cell,
    // u_k = (fl32(x_k - c_k) - o_k) / f with o_k the cell origin in the same
    // centred float32 frame, is within uerr of the truth (coordinate and origin
    // errors 2 ea, three float32 roundings, and the 2^-20-cell slack of the
    // float64 cell assignment of candidate points).  A stencil cell whose
    // farthest corner is within eps (1 - 2^-7) holds only neighbours (float64
    // d2 <= eps2_in, so the box test passes too); one whose nearest face is
    // beyond eps (1 + 2^-7) holds none.  Thresholds are in squared cell units.
    const double inv_m2 = (eps / p.f) * (eps / p.f);
    const double uerr = 4.0 * ea / p.f + 1.0 / 262144.0;               // + 2^-18
    const double mi = 1.0 - 1.0 / 128.0, mo = 1.0 + 1.0 / 128.0;
    p.inv_f32 = __double2float_rn(1.0 / p.f);
    p.uerr = __double2float_ru(uerr);
    p.thr_in = __double2float_rd(inv_m2 * mi * mi * (1.0 - 1.0 / 65536.0));
    p.thr_out = __double2float_ru(inv_m2 * mo * mo * (1.0 + 1.0 / 65536.0));
    p.prune = (!(fl & kFlagNoShortcut) && uerr <= 1.0 / 256.0 && R < 1e30 && e2 > 1e-30) ? 1 : 0;
  }
  p.flags = fl;
  *P = p;
}

// ------------------------------------------------------------------ keys
template <int D, class Key>
__global__ void k_keys(const double* __restrict__ pts, int64_t n, const DevParams* __restrict__ Pp,
                       Key* __restrict__ keys) {
  const DevParams P = *Pp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t key = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      double t = __dmul_rn(__dsub_rn(pts[i * D + k], P.lo[k]), P.inv_f);
      int64_t g = (int64_t)floor(t);
      g = g < 0 ? 0 : (g >= P.G[k] ? P.G[k] - 1 : g);
      key = key * (uint64_t)P.G[k] + (uint64_t)g;
    }
    keys[i] = (Key)key;
  }
}

// sorted structure-of-arrays copy (+ float32 centred copy)
template <int D, bool F32>
__global__ void k_gather(const double* __restrict__ pts, const uint32_t* __restrict__ ids,
                         int64_t n, const DevParams* __restrict__ Pp, double* __restrict__ X,
                         float* __restrict__ Xf) {
  double c[D];
#pragma unroll
  for (int k = 0; k < D; ++k) c[k] = Pp->centre[k];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = ids[i];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      double v = pts[j * D + k];
      X[k * n + i] = v;
      if (F32) Xf[k * n + i] = __double2float_rn(__dsub_rn(v, c[k]));
    }
  }
}

template <class Key>
__global__ void k_run_flags(const Key* __restrict__ keys, int64_t n, uint32_t* __restrict__ fl) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    fl[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

__global__ void k_run_scatter(const uint32_t* __restrict__ fl, const uint32_t* __restrict__ pos,
                              int64_t n, int* __restrict__ reps, const uint32_t* __restrict__ Mdev,
                              unsigned long long* ctr) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (fl[i]) reps[pos[i]] = (int)i;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    reps[*Mdev] = (int)n;
    ctr[kCtrCells] = *Mdev;
  }
}

__global__ void k_cell_counts(const uint32_t* __restrict__ keys, const int* __restrict__ reps,
                              const uint32_t* __restrict__ Mdev, uint32_t* __restrict__ table) {
  const int64_t M = *Mdev;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    int b = reps[m], e = reps[m + 1];
    table[keys[b]] = (uint32_t)(e - b);
  }
}

// sparse grids: hash of the occupied cells, key -> cell index m
__global__ void k_hash_insert(const unsigned long long* __restrict__ keys,
                              const int* __restrict__ reps, const uint32_t* __restrict__ Mdev,
                              unsigned long long* __restrict__ hkeys, uint32_t* __restrict__ hvals,
                              uint32_t mask) {
  const int64_t M = *Mdev;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long k = keys[reps[m]];
    uint32_t h = hash_key(k) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
      unsigned long long prev = atomicCAS(hkeys + h, kHashEmpty, k);
      if (prev == kHashEmpty || prev == k) {
        hvals[h] = (uint32_t)m;
        break;
      }
      h = (h + 1) & mask;
    }
  }
}

// ------------------------------------------------------------- cell helpers
template <int D>
struct CellXYZ {
  int64_t c[3];
};

template <int D>
__device__ __forceinline__ CellXYZ<D> decompose(uint64_t key, const DevParams& P) {
  CellXYZ<D> r;
  uint64_t k = key;
  if (D == 3) {
    r.c[2] = (int64_t)(k % (uint64_t)P.G[2]);
    k /= (uint64_t)P.G[2];
  } else {
    r.c[2] = 0;
  }
  r.c[1] = (int64_t)(k % (uint64_t)P.G[1]);
  r.c[0] = (int64_t)(k / (uint64_t)P.G[1]);
  return r;
}

// key of cell (c + o), or -1 when outside the grid
template <int D>
__device__ __forceinline__ int64_t offset_key(const CellXYZ<D>& c, int ox, int oy, int oz,
                                              const DevParams& P) {
  int64_t x = c.c[0] + ox, y = c.c[1] + oy;
  if (x < 0 || x >= P.G[0] || y < 0 || y >= P.G[1]) return -1;
  int64_t k = x * P.G[1] + y;
  if (D == 3) {
    int64_t z = c.c[2] + oz;
    if (z < 0 || z >= P.G[2]) return -1;
    k = k * P.G[2] + z;
  }
  return k;
}


// Loads one candidate (sorted position q) in the layout the mode tests with.
template <int D, bool F32>
struct Cand {
  double x[D];
  float f[D];
};

template <int D, bool F32>
__device__ __forceinline__ void load_cand(Cand<D, F32>& c, const double* __restrict__ X,
                                          const float* __restrict__ Xf, int64_t n, int64_t q) {
#pragma unroll
  for (int k = 0; k < D; ++k) {
    if (F32) c.f[k] = Xf[k * n + q];
    else c.x[k] = X[k * n + q];
  }
}

// Per-warp staging of up to 32 "A" points (the points of the cell in work).
template <int D>
struct WarpStage {
  double x[32][D];
  float f[32][D];
};

struct Tally {
  uint32_t t64 = 0, t32 = 0, band = 0, asym = 0;
};

// float32 distance (centred copies); FMA-rounded as the band derivation assumes
template <int D>
__device__ __forceinline__ float dist2_f32(const float* a, const float* b) {
  float u = __fsub_rn(a[0], b[0]);
  float s = __fmul_rn(u, u);
  float v = __fsub_rn(a[1], b[1]);
  s = __fmaf_rn(v, v, s);
  if (D == 3) {
    float w = __fsub_rn(a[2], b[2]);
    s = __fmaf_rn(w, w, s);
  }
  return s;
}

// Directed test "cand is a neighbour of centre".  One side is a staged point
// (coords in smem), the other a candidate (coords in registers / memory).
// stage_is_centre selects which is the centre of the query box.
template <int D, bool F32>
__device__ __forceinline__ bool pair_test(const double* sx, const float* sf, const Cand<D, F32>& c,
                                          const double* __restrict__ X, int64_t n, int64_t q,
                                          bool stage_is_centre, const DevParams& P, Tally& t) {
  if (F32) {
    ++t.t32;
    float s = dist2_f32<D>(sf, c.f);
    if (s < P.eps2_lo32) return true;
    if (s > P.eps2_hi32) return false;
    ++t.band;
    double qx[D];
#pragma unroll
    for (int k = 0; k < D; ++k) qx[k] = X[k * n + q];
    ++t.t64;
    double d2 = dist2_f64<D>(sx, qx);
    return stage_is_centre ? pred_from_d2<D>(d2, sx, qx, P) : pred_from_d2<D>(d2, qx, sx, P);
  } else {
    ++t.t64;
    double d2 = dist2_f64<D>(sx, c.x);
    return stage_is_centre ? pred_from_d2<D>(d2, sx, c.x, P) : pred_from_d2<D>(d2, c.x, sx, P);
  }
}

// Symmetric test for core-core links: true when the pair is a neighbour in both
// directions; counts pairs that are neighbours in exactly one direction.
template <int D, bool F32>
__device__ __forceinline__ bool link_test(const double* sx, const float* sf, const Cand<D, F32>& c,
                                          const double* __restrict__ X, int64_t n, int a, int q,
                                          const DevParams& P, Tally& t,
                                          int* __restrict__ asym_list, unsigned long long* ctr) {
  double qx[D];
  if (F32) {
    ++t.t32;
    float s = dist2_f32<D>(sf, c.f);
    if (s < P.eps2_lo32) return true;
    if (s > P.eps2_hi32) return false;
    ++t.band;
#pragma unroll
    for (int k = 0; k < D; ++k) qx[k] = X[k * n + q];
  } else {
#pragma unroll
    for (int k = 0; k < D; ++k) qx[k] = c.x[k];
  }
  ++t.t64;
  double d2 = dist2_f64<D>(sx, qx);
  if (d2 <= P.eps2_in) return true;
  if (!(d2 <= P.eps2)) return false;
  bool f = box_f64<D>(sx, qx, P.eps), b = box_f64<D>(qx, sx, P.eps);
  if (f != b) {
    // q is a neighbour of a but not a of q (f), or the reverse: a directed
    // link that the merge replay (k_asym_resolve) needs.
    ++t.asym;
    unsigned long long slot = atomicAdd(ctr + kCtrAsymEdges, 1ull);
    if (slot < (unsigned long long)kAsymCap) {
      asym_list[2 * slot] = f ? a : q;
      asym_list[2 * slot + 1] = f ? q : a;
    }
  }
  return f && b;
}

__device__ __forceinline__ void flush_tally(const Tally& t, unsigned long long* ctr) {
  // one atomic per warp per counter
  unsigned long long a = t.t64, b = t.t32, c = t.band, d = t.asym;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(kFull, a, o);
    b += __shfl_xor_sync(kFull, b, o);
    c += __shfl_xor_sync(kFull, c, o);
    d += __shfl_xor_sync(kFull, d, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (a) atomicAdd(ctr + kCtrTests64, a);
    if (b) atomicAdd(ctr + kCtrTests32, b);
    if (c) atomicAdd(ctr + kCtrBand, c);
    if (d) atomicAdd(ctr + kCtrAsym, d);
  }
}

__device__ __forceinline__ int warp_min_i32(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// Cell lookup.  Dense grids: the cell table gives every cell's point range.
// Sparse grids: a hash of the occupied cells' keys gives the cell index m, and
// reps[m]..reps[m+1] its points.  The probe loop is bounded by the table size.
template <bool SPARSE>
struct GridView {
  const uint32_t* start;
  const unsigned long long* hkeys;
  const uint32_t* hvals;
  const int* reps;
  uint32_t hmask;

  __device__ __forceinline__ int find(uint64_t k) const {
    uint32_t h = hash_key(k) & hmask;
    for (uint32_t probe = 0; probe <= hmask; ++probe) {
      unsigned long long kk = hkeys[h];
      if (kk == k) return (int)hvals[h];
      if (kk == kHashEmpty) return -1;
      h = (h + 1) & hmask;
    }
    return -1;
  }
  // points of cell k: [x, y)
  __device__ __forceinline__ int2 cell(uint64_t k) const {
    if (!SPARSE) return make_int2((int)start[k], (int)start[k + 1]);
    int m = find(k);
    return m < 0 ? make_int2(0, 0) : make_int2(reps[m], reps[m + 1]);
  }
  // points of the cells k0..k1 (consecutive keys along one row): one contiguous
  // range, because no other key sorts between them
  __device__ __forceinline__ int2 span(uint64_t k0, uint64_t k1) const {
    if (!SPARSE) return make_int2((int)start[k0], (int)start[k1 + 1]);
    int lo = INT_MAX, hi = 0;
    for (uint64_t k = k0; k <= k1; ++k) {
      int m = find(k);
      if (m >= 0) {
        lo = min(lo, reps[m]);
        hi = max(hi, reps[m + 1]);
      }
    }
    return lo == INT_MAX ? make_int2(0, 0) : make_int2(lo, hi);
  }
};

template <bool SPARSE>
__host__ __device__ __forceinline__ GridView<SPARSE> view_of(const gdl::Bufs& B) {
  return GridView<SPARSE>{B.start, B.hkeys, B.hvals, B.reps, B.hmask};
}

template <bool SPARSE>
__device__ __forceinline__ uint64_t key_at(const gdl::Bufs& B, int64_t i) {
  if (SPARSE) return static_cast<const unsigned long long*>(B.keys)[i];
  return static_cast<const uint32_t*>(B.keys)[i];
}

// first sorted position (rep) of the cell holding sorted position i
__device__ __forceinline__ int rep_of(const gdl::Bufs& B, int64_t i) {
  return B.reps[B.runpos[i] + B.runfl[i] - 1];
}


// ------------------------------------------------------------ stencil tables
// Offsets within +-2 cells, built at compile time.  kRows: the (ox, oy) rows a
// core count scans, own row first.  kHalf[d][pass]: the half stencil (o > 0
// lexicographically) split into near offsets (all |o_k| <= 1, pass 0) and the
// rest (pass 1).  kFull[d]: all offsets (border search).
struct OffTab {
  signed char o[128][3];
  int n;
};

constexpr OffTab make_rows(int D) {
  OffTab t{};
  const int order[5] = {0, -1, 1, -2, 2};
  for (int a = 0; a < 5; ++a)
    for (int b = 0; b < (D == 3 ? 5 : 1); ++b) {
      t.o[t.n][0] = (signed char)order[a];
      t.o[t.n][1] = (signed char)(D == 3 ? order[b] : 0);
      t.o[t.n][2] = 0;
      ++t.n;
    }
  return t;
}

constexpr OffTab make_half(int D, int pass) {
  OffTab t{};
  const int zr = D == 3 ? 2 : 0;
  for (int x = -2; x <= 2; ++x)
    for (int y = -2; y <= 2; ++y)
      for (int z = -zr; z <= zr; ++z) {
        bool pos = x > 0 || (x == 0 && (y > 0 || (y == 0 && z > 0)));
        bool near = x >= -1 && x <= 1 && y >= -1 && y <= 1 && z >= -1 && z <= 1;
        if (!pos || (pass == 0) != near) continue;
        t.o[t.n][0] = (signed char)x;
        t.o[t.n][1] = (signed char)y;
        t.o[t.n][2] = (signed char)z;
        ++t.n;
      }
  return t;
}

constexpr OffTab make_full(int D) {
  OffTab t{};
  const int zr = D == 3 ? 2 : 0;
  for (int x = -2; x <= 2; ++x)
    for (int y = -2; y <= 2; ++y)
      for (int z = -zr; z <= zr; ++z) {
        t.o[t.n][0] = (signed char)x;
        t.o[t.n][1] = (signed char)y;
        t.o[t.n][2] = (signed char)z;
        ++t.n;
      }
  return t;
}

__constant__ OffTab kRows[2] = {make_rows(2), make_rows(3)};
__constant__ OffTab kHalf[2][2] = {{make_half(2, 0), make_half(2, 1)},
                                   {make_half(3, 0), make_half(3, 1)}};
__constant__ OffTab kFullSt[2] = {make_full(2), make_full(3)};

// Per-warp list of candidate rows: row r holds the points lo[r] .. lo[r]+len,
// and pre[r] is the exclusive prefix of the lengths (rows concatenated in
// table order).  Lane r looks its row up, so all lookups are in flight at once.
struct RowList {
  int lo[32];
  int pre[32];
};

template <int D, bool SPARSE>
__device__ __forceinline__ int build_rows(RowList& RL, const GridView<SPARSE>& gv,
                                          const CellXYZ<D>& cc, const DevParams& P, int lane) {
  const OffTab& T = kRows[D - 2];
  const int64_t Gl = P.G[D - 1];
  const int64_t cl = cc.c[D - 1];
  const int64_t l0 = cl - 2 < 0 ? 0 : cl - 2;
  const int64_t l1 = cl + 2 >= Gl ? Gl - 1 : cl + 2;
  int lo = 0, len = 0;
  if (lane < T.n) {
    int64_t rowkey = offset_key<D>(cc, T.o[lane][0], T.o[lane][1], 0, P);
    if (rowkey >= 0) {
      rowkey -= cl;
      const int2 rg = gv.span((uint64_t)(rowkey + l0), (uint64_t)(rowkey + l1));
      lo = rg.x;
      len = rg.y - rg.x;
    }
  }
  int inc = len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += v;
  }
  RL.lo[lane] = lo;
  RL.pre[lane] = inc - len;
  __syncwarp();
  return __shfl_sync(kFull, inc, 31);
}

// sorted position of concatenated candidate c (0 <= c < total)
__device__ __forceinline__ int row_pos(const RowList& RL, int nrows, int c) {
  int r = 0;
#pragma unroll
  for (int step = 16; step; step >>= 1)
    if (r + step < nrows && RL.pre[r + step] <= c) r += step;
  return RL.lo[r] + (c - RL.pre[r]);
}

constexpr int kWarpsPerBlock = 8;
constexpr int kCellThreads = kWarpsPerBlock * 32;

// ----------------------------------------------- cell-level classification
// Origin (low corner) of cell cc in the centred float32 frame.
template <int D>
__device__ __forceinline__ void cell_origin32(const CellXYZ<D>& cc, const DevParams& P, float* o) {
#pragma unroll
  for (int k = 0; k < D; ++k)
    o[k] = __double2float_rn(
        __dsub_rn(__dadd_rn(P.lo[k], __dmul_rn((double)cc.c[k], P.f)), P.centre[k]));
}

// A point's position inside its own cell, in cell units (error <= P.uerr).
template <int D>
__device__ __forceinline__ void frac_pos(const float* xf, const float* o, const DevParams& P,
                                         float* u) {
#pragma unroll
  for (int k = 0; k < D; ++k) u[k] = __fmul_rn(__fsub_rn(xf[k], o[k]), P.inv_f32);
}

// Cell at offset (ox, oy, oz) from the point's cell: 1 every point in it is a
// neighbour (both ways), -1 none is, 0 must be tested.
template <int D>
__device__ __forceinline__ int classify(const float* u, int ox, int oy, int oz,
                                        const DevParams& P) {
  const int off[3] = {ox, oy, oz};
  float smax = 0.0f, smin = 0.0f;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const float a = u[k] - (float)off[k];  // position relative to the box [off, off + 1]
    const float b = a - 1.0f;
    const float mx = fmaxf(fabsf(a), fabsf(b)) + P.uerr;
    const float mn = fmaxf(fmaxf(-a, b) - P.uerr, 0.0f);
    smax = fmaf(mx, mx, smax);
    smin = fmaf(mn, mn, smin);
  }
  if (smax <= P.thr_in) return 1;
  if (smin >= P.thr_out) return -1;
  return 0;
}

// ------------------------------------------------- thread-per-cell front ends
// Most cells need little work: isolated noise points whose stencil holds fewer
// than minpts points, cells whose neighbour links are found by the first test,
// border points with a handful of candidate cores.  The *_scan kernels give one
// thread to each cell and finish those cases inline (bounded work per thread);
// a cell that needs more is appended to the heavy list and handled by the
// warp-cooperative *_heavy kernel that follows.
constexpr int kScanThreadsPerBlock = 256;
constexpr int kInlineCoreTests = 160;    // points x candidates done by one thread
constexpr int kInlineLinkTests = 48;     // tests before a link search goes to a warp
constexpr int kInlineBorderTests = 160;  // non-core points x candidate cores

// warp-aggregated append to the heavy list (all 32 lanes must call it)
__device__ __forceinline__ void heavy_push(const gdl::Bufs& B, int slot, bool push, int64_t m,
                                           unsigned long long mask) {
  const unsigned bal = __ballot_sync(kFull, push);
  if (!bal) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(bal) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(B.ctr + slot, (unsigned long long)__popc(bal));
  base = __shfl_sync(kFull, base, leader);
  if (push) {
    const unsigned long long at = base + (unsigned long long)__popc(bal & ((1u << lane) - 1u));
    B.hv_cell[at] = (int)m;
    B.hv_mask[at] = mask;
  }
}

template <int D, bool F32>
__device__ __forceinline__ void load_point(double* x, float* f, const gdl::Bufs& B, int64_t n,
                                           int64_t i, bool prune) {
#pragma unroll
  for (int k = 0; k < D; ++k) {
    x[k] = B.X[k * n + i];
    if (F32 || prune) f[k] = B.Xf[k * n + i];
  }
}

template <int D, bool F32, bool SPARSE>
__global__ void __launch_bounds__(kScanThreadsPerBlock) k_core_scan(const gdl::Bufs B, int64_t n) {
  __shared__ DevParams sP;
  if (threadIdx.x == 0) sP = *B.P;
  __syncthreads();
  const DevParams& P = sP;
  const GridView<SPARSE> gv = view_of<SPARSE>(B);
  const OffTab& T = kRows[D - 2];
  const int lane = threadIdx.x & 31;
  const bool prune = P.prune != 0;
  const int64_t M = *B.M;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  Tally t;
  for (int64_t m0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); m0 < M; m0 += stride) {
    const int64_t m = m0 + lane;
    bool push = false;
    if (m < M) {
      const int b = B.reps[m], e = B.reps[m + 1], sz = e - b;
      if (sz >= P.minpts) {
        push = true;  // dense: the warp kernel marks it
      } else {
        const CellXYZ<D> cc = decompose<D>(key_at<SPARSE>(B, b), P);
        const int64_t Gl = P.G[D - 1], cl = cc.c[D - 1];
        const int64_t l0 = cl - 2 < 0 ? 0 : cl - 2;
        const int64_t l1 = cl + 2 >= Gl ? Gl - 1 : cl + 2;
        int total = 0;
        for (int r = 0; r < T.n; ++r) {
          int64_t rowkey = offset_key<D>(cc, T.o[r][0], T.o[r][1], 0, P);
          if (rowkey < 0) continue;
          rowkey -= cl;
          const int2 rg = gv.span((uint64_t)(rowkey + l0), (uint64_t)(rowkey + l1));
          total += rg.y - rg.x;
        }
        int ncore = 0, mn = INT_MAX;
        if (total >= P.minpts) {
          float o[D];
          if (prune) cell_origin32<D>(cc, P, o);
          for (int i = b; i < e && !push; ++i) {
            double px[D];
            float pf[D], u[D];
            load_point<D, F32>(px, pf, B, n, i, prune);
            if (prune) frac_pos<D>(pf, o, P, u);
            // pass 1: cells wholly inside count without a test; sum the rest
            int cnt = 0, ptot = total;
            if (prune) {
              ptot = 0;
              for (int r = 0; r < T.n; ++r) {
                int64_t rowkey = offset_key<D>(cc, T.o[r][0], T.o[r][1], 0, P);
                if (rowkey < 0) continue;
                rowkey -= cl;
                for (int64_t z = l0; z <= l1; ++z) {
                  const int2 c = gv.cell((uint64_t)(rowkey + z));
                  if (c.x == c.y) continue;
                  const int d = (int)(z - cl);
                  const int cls = D == 3 ? classify<D>(u, T.o[r][0], T.o[r][1], d, P)
                                         : classify<D>(u, T.o[r][0], d, 0, P);
                  if (cls > 0) cnt += c.y - c.x;
                  else if (cls == 0) ptot += c.y - c.x;
                }
              }
            }
            if (cnt < P.minpts && cnt + ptot >= P.minpts) {
              if (ptot > kInlineCoreTests) {
                push = true;  // too many candidates for one thread
                break;
              }
              // pass 2: test the undecided cells
              for (int r = 0; r < T.n && cnt < P.minpts; ++r) {
                int64_t rowkey = offset_key<D>(cc, T.o[r][0], T.o[r][1], 0, P);
                if (rowkey < 0) continue;
                rowkey -= cl;
                for (int64_t z = l0; z <= l1 && cnt < P.minpts; ++z) {
                  const int2 c = gv.cell((uint64_t)(rowkey + z));
                  if (c.x == c.y) continue;
                  if (prune) {
                    const int d = (int)(z - cl);
                    const int cls = D == 3 ? classify<D>(u, T.o[r][0], T.o[r][1], d, P)
                                           : classify<D>(u, T.o[r][0], d, 0, P);
                    if (cls != 0) continue;
                  }
                  for (int q = c.x; q < c.y && cnt < P.minpts; ++q) {
                    Cand<D, F32> cd;
                    load_cand<D, F32>(cd, B.X, B.Xf, n, q);
                    cnt += pair_test<D, F32>(px, pf, cd, B.X, n, q, true, P, t) ? 1 : 0;
                  }
                }
              }
            }
            const bool isc = cnt >= P.minpts;
            B.core[i] = isc ? 1 : 0;
            if (isc) {
              ++ncore;
              mn = min(mn, (int)B.ids[i]);
            }
          }
        } else {
          for (int i = b; i < e; ++i) B.core[i] = 0;  // fewer candidates than minpts
        }
        if (!push) {
          B.cellcore[b] = ncore;
          B.cellmin[b] = mn;
        }
      }
    }
    heavy_push(B, kCtrHeavyCore, push, m, 0);
  }
  flush_tally(t, B.ctr);
}

// Bounded link search between the core points of cells A and B by one thread:
// 1 found (neighbours both ways), 0 none exists, -1 budget spent.  With cell
// classification, a core point of A that has all of B within reach links at
// once (B holds a core point), and one that has none of B in reach is skipped.
template <int D, bool F32>
__device__ __forceinline__ int inline_link(const gdl::Bufs& B, int64_t n, int bA, int eA, int bB,
                                           int eB, const float* oA, int ox, int oy, int oz,
                                           const DevParams& P, Tally& t) {
  const bool prune = P.prune != 0;
  int budget = kInlineLinkTests;
  bool skipped = false;
  for (int a = bA; a < eA; ++a) {
    if (!B.core[a]) continue;
    double ax[D];
    float af[D];
    load_point<D, F32>(ax, af, B, n, a, prune);
    if (prune) {
      float u[D];
      frac_pos<D>(af, oA, P, u);
      const int cls = classify<D>(u, ox, oy, oz, P);
      if (cls > 0) return 1;
      if (cls < 0) continue;
    }
    for (int q = bB; q < eB; ++q) {
      if (!B.core[q]) continue;
      if (budget-- == 0) return -1;
      Cand<D, F32> cd;
      load_cand<D, F32>(cd, B.X, B.Xf, n, q);
      if (link_test<D, F32>(ax, af, cd, B.X, n, a, q, P, t, B.asym, B.ctr)) return 1;
    }
  }
  (void)skipped;
  return 0;
}

template <int D, bool F32, bool SPARSE>
__global__ void __launch_bounds__(kScanThreadsPerBlock)
k_union_scan(const gdl::Bufs B, int64_t n, int pass) {
  __shared__ DevParams sP;
  if (threadIdx.x == 0) sP = *B.P;
  __syncthreads();
  const DevParams& P = sP;
  const GridView<SPARSE> gv = view_of<SPARSE>(B);
  const OffTab& T = kHalf[D - 2][pass];
  const int lane = threadIdx.x & 31;
  const int64_t M = *B.M;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  Tally t;
  for (int64_t m0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); m0 < M; m0 += stride) {
    const int64_t m = m0 + lane;
    unsigned long long open = 0;
    if (m < M) {
      const int b = B.reps[m];
      if (B.cellcore[b] > 0) {
        const int e = B.reps[m + 1];
        const CellXYZ<D> cc = decompose<D>(key_at<SPARSE>(B, b), P);
        float oA[D];
        if (P.prune) cell_origin32<D>(cc, P, oA);
        for (int tt = 0; tt < T.n; ++tt) {
          const int64_t kb = offset_key<D>(cc, T.o[tt][0], T.o[tt][1], T.o[tt][2], P);
          if (kb < 0) continue;
          const int2 cb = gv.cell((uint64_t)kb);
          if (cb.x == cb.y || B.cellcore[cb.x] == 0) continue;
          if (uf_find(B.parent, b) == uf_find(B.parent, cb.x)) continue;
          const int r = inline_link<D, F32>(B, n, b, e, cb.x, cb.y, oA, T.o[tt][0], T.o[tt][1],
                                            T.o[tt][2], P, t);
          if (r > 0) uf_union(B.parent, B.cellmin, b, cb.x);
          else if (r < 0) open |= 1ull << tt;
        }
      }
    }
    heavy_push(B, kCtrHeavyUnion, open != 0, m, open);
  }
  flush_tally(t, B.ctr);
}

template <int D, bool F32, bool SPARSE>
__global__ void __launch_bounds__(kScanThreadsPerBlock) k_border_scan(const gdl::Bufs B, int64_t n) {
  __shared__ DevParams sP;
  if (threadIdx.x == 0) sP = *B.P;
  __syncthreads();
  const DevParams& P = sP;
  const GridView<SPARSE> gv = view_of<SPARSE>(B);
  const OffTab& T = kFullSt[D - 2];
  const int lane = threadIdx.x & 31;
  const bool prune = P.prune != 0;
  const int64_t M = *B.M;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  Tally t;
  for (int64_t m0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); m0 < M; m0 += stride) {
    const int64_t m = m0 + lane;
    bool push = false;
    if (m < M) {
      const int b = B.reps[m], e = B.reps[m + 1];
      const int nnc = (e - b) - B.cellcore[b];
      if (nnc > 0) {
        const CellXYZ<D> cc = decompose<D>(key_at<SPARSE>(B, b), P);
        int cores = 0;
        for (int tt = 0; tt < T.n; ++tt) {
          const int64_t kb = offset_key<D>(cc, T.o[tt][0], T.o[tt][1], T.o[tt][2], P);
          if (kb < 0) continue;
          const int2 cb = gv.cell((uint64_t)kb);
          if (cb.x < cb.y) cores += B.cellcore[cb.x];
        }
        if (cores > 0) {
          // no core point in reach: the non-core points stay NOISE (else below)
          float o[D];
          if (prune) cell_origin32<D>(cc, P, o);
          int budget = kInlineBorderTests;
          for (int i = b; i < e && !push; ++i) {
            if (B.core[i]) continue;
            double px[D];
            float pf[D], u[D];
            load_point<D, F32>(px, pf, B, n, i, prune);
            if (prune) frac_pos<D>(pf, o, P, u);
            int best = INT_MAX;
            for (int tt = 0; tt < T.n && !push; ++tt) {
              const int64_t kb = offset_key<D>(cc, T.o[tt][0], T.o[tt][1], T.o[tt][2], P);
              if (kb < 0) continue;
              const int2 cb = gv.cell((uint64_t)kb);
              if (cb.x == cb.y || B.cellcore[cb.x] == 0) continue;
              const int cB = B.cellcid[cb.x];
              if (cB >= best) continue;
              if (prune) {
                const int cls = classify<D>(u, T.o[tt][0], T.o[tt][1], T.o[tt][2], P);
                if (cls > 0) {
                  best = cB;  // every point of that cell, a core among them, is in reach
                  continue;
                }
                if (cls < 0) continue;
              }
              for (int q = cb.x; q < cb.y; ++q) {
                if (!B.core[q]) continue;
                if (budget-- == 0) {
                  push = true;  // too much for one thread
                  break;
                }
                Cand<D, F32> cd;
                load_cand<D, F32>(cd, B.X, B.Xf, n, q);
                if (pair_test<D, F32>(px, pf, cd, B.X, n, q, false, P, t)) {
                  best = cB;
                  break;
                }
              }
            }
            if (!push && best != INT_MAX) B.lab[i] = best;
          }
        }
      }
    }
    heavy_push(B, kCtrHeavyBorder, push, m, 0);
  }
  flush_tally(t, B.ctr);
}

// ------------------------------------------------------------- core flags
// One warp per non-empty cell.  Dense cells are all core.  Otherwise the warp
// looks up its candidate rows (5 cells along the last axis each, 5 rows in 2D,
// 25 in 3D; one lane per row), concatenates them, and streams the candidates
// 32 at a time, one per lane.  Each staged point p of the cell gets
// __ballot_sync + __popc of the lanes holding a neighbour.  The warp stops as
// soon as every staged p has reached minpts (own row first, so dense
// neighbourhoods stop after one tile).
template <int D, bool F32, bool SPARSE>
__global__ void __launch_bounds__(kCellThreads) k_core_heavy(const gdl::Bufs B, int64_t n) {
  __shared__ DevParams sP;
  __shared__ WarpStage<D> stage[kWarpsPerBlock];
  __shared__ RowList rows[kWarpsPerBlock];
  if (threadIdx.x == 0) sP = *B.P;
  __syncthreads();
  const DevParams& P = sP;
  const GridView<SPARSE> gv = view_of<SPARSE>(B);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  WarpStage<D>& S = stage[w];
  RowList& RL = rows[w];
  const int nrows = kRows[D - 2].n;
  const double* __restrict__ X = B.X;
  const float* __restrict__ Xf = B.Xf;
    const int64_t W = (int64_t)gridDim.x * kWarpsPerBlock;
  Tally t;
  unsigned long long dense = 0;
  const int64_t H = (int64_t)B.ctr[kCtrHeavyCore];
  for (int64_t h = (int64_t)blockIdx.x * kWarpsPerBlock + w; h < H; h += W) {
    const int64_t m = B.hv_cell[h];
    const int b = B.reps[m], e = B.reps[m + 1], sz = e - b;
    if (sz >= P.minpts) {
      int mn = INT_MAX;
      for (int i = b + lane; i < e; i += 32) {
        B.core[i] = 1;
        mn = min(mn, (int)B.ids[i]);
      }
      mn = warp_min_i32(mn);
      if (lane == 0) { B.cellcore[b] = sz; B.cellmin[b] = mn; ++dense; }
      continue;
    }
    const CellXYZ<D> cc = decompose<D>(key_at<SPARSE>(B, b), P);
    const int total = build_rows<D, SPARSE>(RL, gv, cc, P, lane);
    int ncore = 0, mn = INT_MAX;
    for (int c0 = 0; c0 < sz; c0 += 32) {
      const int na = min(32, sz - c0);
      if (lane < na) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
          S.x[lane][k] = X[k * n + b + c0 + lane];
          if (F32) S.f[lane][k] = Xf[k * n + b + c0 + lane];
        }
      }
      __syncwarp();
      int mycnt = 0;
      bool done = false;
      for (int base = 0; base < total && !done; base += 32) {
        const int c = base + lane;
        const bool valid = c < total;
        int q = 0;
        Cand<D, F32> cd;
        if (valid) {
          q = row_pos(RL, nrows, c);
          load_cand<D, F32>(cd, X, Xf, n, q);
        }
        for (int j = 0; j < na; ++j) {
          bool hit = valid && pair_test<D, F32>(S.x[j], S.f[j], cd, X, n, q, true, P, t);
          unsigned bal = __ballot_sync(kFull, hit);
          if (lane == j) mycnt += __popc(bal);
        }
        done = __all_sync(kFull, lane >= na || mycnt >= P.minpts);
      }
      const bool isc = lane < na && mycnt >= P.minpts;
      if (lane < na) B.core[b + c0 + lane] = isc ? 1 : 0;
      if (isc) mn = min(mn, (int)B.ids[b + c0 + lane]);
      ncore += __popc(__ballot_sync(kFull, isc));
      __syncwarp();
    }
    mn = warp_min_i32(mn);
    if (lane == 0) { B.cellcore[b] = ncore; B.cellmin[b] = mn; }
  }
  flush_tally(t, B.ctr);
  if (lane == 0 && dense) atomicAdd(B.ctr + kCtrDenseCells, dense);
}

// ------------------------------------------------------------- union-find
__global__ void k_parent_init(const gdl::Bufs B) {
  const int64_t M = *B.M;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    int b = B.reps[m];
    B.parent[b] = b;
  }
}

// One warp per cell A with core points.  Lanes look up the half-stencil
// neighbour cells of this pass in parallel (pass 0: offsets within +-1, pass 1:
// the rest -- running the near pass first lets most far pairs be skipped
// because their cells are already in one component).  For each neighbour B
// with core points in another component, the warp looks for one core-core pair
// that are neighbours both ways (lanes over B's points, A's core points
// broadcast) and unites the two cells.
template <int D, bool F32, bool SPARSE>
__global__ void __launch_bounds__(kCellThreads) k_union_heavy(const gdl::Bufs B, int64_t n, int pass) {
  __shared__ DevParams sP;
  if (threadIdx.x == 0) sP = *B.P;
  __syncthreads();
  const DevParams& P = sP;
  const GridView<SPARSE> gv = view_of<SPARSE>(B);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const double* __restrict__ X = B.X;
  const float* __restrict__ Xf = B.Xf;
    const int64_t W = (int64_t)gridDim.x * kWarpsPerBlock;
  const OffTab& T = kHalf[D - 2][pass];
  Tally t;
  const int64_t H = (int64_t)B.ctr[kCtrHeavyUnion];
  for (int64_t h = (int64_t)blockIdx.x * kWarpsPerBlock + w; h < H; h += W) {
    const int64_t m = B.hv_cell[h];
    const unsigned long long open = B.hv_mask[h];
    const int b = B.reps[m];
    const int e = B.reps[m + 1];
    const CellXYZ<D> cc = decompose<D>(key_at<SPARSE>(B, b), P);
    for (int t0 = 0; t0 < T.n; t0 += 32) {
      const int tt = t0 + lane;
      bool cand = false;
      int bB = 0, eB = 0;
      if (tt < T.n && ((open >> tt) & 1ull)) {
        const int64_t kb = offset_key<D>(cc, T.o[tt][0], T.o[tt][1], T.o[tt][2], P);
        if (kb >= 0) {
          const int2 cb = gv.cell((uint64_t)kb);
          bB = cb.x;
          eB = cb.y;
          cand = bB < eB && B.cellcore[bB] > 0 && uf_find(B.parent, bB) != uf_find(B.parent, b);
        }
      }
      unsigned mask = __ballot_sync(kFull, cand);
      while (mask) {
        const int src = __ffs(mask) - 1;
        mask &= mask - 1;
        const int cbB = __shfl_sync(kFull, bB, src);
        const int ceB = __shfl_sync(kFull, eB, src);
        if (uf_find(B.parent, b) == uf_find(B.parent, cbB)) continue;
        bool found = false;
        for (int qb = cbB; qb < ceB && !found; qb += 32) {
          const int q = qb + lane;
          const bool valid = q < ceB && B.core[q];
          Cand<D, F32> c;
          if (valid) load_cand<D, F32>(c, X, Xf, n, q);
          for (int a = b; a < e && !found; ++a) {
            if (!B.core[a]) continue;
            double ax[D];
            float af[D];
#pragma unroll
            for (int k = 0; k < D; ++k) {
              ax[k] = X[k * n + a];
              if (F32) af[k] = Xf[k * n + a];
            }
            bool hit = valid && link_test<D, F32>(ax, af, c, X, n, a, q, P, t, B.asym, B.ctr);
            found = __any_sync(kFull, hit);
          }
        }
        if (found && lane == 0) uf_union(B.parent, B.cellmin, b, cbB);
        __syncwarp();
      }
    }
  }
  flush_tally(t, B.ctr);
}

// Merge replay for one-directional core links.  Components of the symmetric
// core graph are what the reference's sequential expansion produces when every
// core-core neighbour relation is mutual.  When core a has core b in its
// neighbourhood but not the reverse (the query box and the distance test can
// disagree in the last bit), the reference's scan (dbscan_rtree_exp.cpp:363-404)
// lets the cluster that expands a swallow b's component if that component is
// still unvisited -- which depends on the order clusters open.  This kernel
// replays exactly that order over the few components touched by such links:
// components in order of their smallest core index; each unassigned one opens
// a cluster that absorbs every unassigned component reachable along directed
// links.  Absorbed roots are re-parented under the opening root.  One thread;
// the list holds at most kAsymCap links (more is reported as an error).
__global__ void k_asym_resolve(const gdl::Bufs B) {
  const int* __restrict__ cellmin = B.cellmin;
  int* parent = B.parent;
  const int* __restrict__ asym_list = B.asym;
  unsigned long long* ctr = B.ctr;
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long E = ctr[kCtrAsymEdges];
  if (E == 0) return;
  if (E > (unsigned long long)kAsymCap) return;  // reported by the host
  __shared__ int from[kAsymCap], to[kAsymCap];
  __shared__ int node[2 * kAsymCap], assigned[2 * kAsymCap];
  int ne = 0, nv = 0;
  for (unsigned long long i = 0; i < E; ++i) {
    int a = asym_list[2 * i], b = asym_list[2 * i + 1];
    int ra = uf_find(parent, rep_of(B, a));
    int rb = uf_find(parent, rep_of(B, b));
    if (ra == rb) continue;
    from[ne] = ra;
    to[ne] = rb;
    ++ne;
    int r2[2] = {ra, rb};
    for (int k = 0; k < 2; ++k) {
      bool seen = false;
      for (int v = 0; v < nv && !seen; ++v) seen = node[v] == r2[k];
      if (!seen) node[nv++] = r2[k];
    }
  }
  // order the components by smallest core index (insertion sort, small)
  for (int i = 1; i < nv; ++i) {
    int x = node[i], j = i - 1;
    while (j >= 0 && cellmin[node[j]] > cellmin[x]) { node[j + 1] = node[j]; --j; }
    node[j + 1] = x;
  }
  // links as indices into the ordered node list
  for (int e = 0; e < ne; ++e) {
    int fi = 0, ti = 0;
    for (int u = 0; u < nv; ++u) {
      if (node[u] == from[e]) fi = u;
      if (node[u] == to[e]) ti = u;
    }
    from[e] = fi;
    to[e] = ti;
  }
  for (int v = 0; v < nv; ++v) assigned[v] = -1;
  for (int v = 0; v < nv; ++v) {
    if (assigned[v] >= 0) continue;
    assigned[v] = node[v];
    // grow the opened cluster along directed links until nothing changes
    bool grew = true;
    while (grew) {
      grew = false;
      for (int e = 0; e < ne; ++e) {
        if (assigned[from[e]] == node[v] && assigned[to[e]] < 0) {
          assigned[to[e]] = node[v];
          grew = true;
        }
      }
    }
  }
  for (int v = 0; v < nv; ++v)
    if (assigned[v] != node[v]) parent[node[v]] = assigned[v];
}

// parent[b] <- root (full path compression)
__global__ void k_compress(const gdl::Bufs B) {
  const int64_t M = *B.M;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    const int b = B.reps[m];
    if (B.cellcore[b] == 0) continue;
    B.parent[b] = uf_find(B.parent, b);
  }
}

// every root flags its component's smallest core index
__global__ void k_roots(const gdl::Bufs B) {
  const int64_t M = *B.M;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    const int b = B.reps[m];
    if (B.cellcore[b] == 0) continue;
    if (uf_find(B.parent, b) == b) B.Fmark[B.cellmin[b]] = 1u;
  }
}

// Cluster id of every cell with core points (ordered by smallest core index:
// Fmark now holds the exclusive scan of the root marks over original indices),
// and the provisional label of every point: its cluster if core, NOISE otherwise.
__global__ void k_label(const gdl::Bufs B, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int b = rep_of(B, i);
    int cl = INT_MAX;
    if (B.cellcore[b] > 0) cl = (int)B.Fmark[B.cellmin[uf_find(B.parent, b)]];
    if (i == b) B.cellcid[b] = cl;
    B.lab[i] = B.core[i] ? cl : kNoise;
  }
}

// Border points: one warp per cell with non-core points (only non-dense cells
// have any).  Each staged non-core point takes the smallest cluster id among
// the cells whose core points have it in their neighbourhood (centre = the core
// point, as the reference's expansion queries from the core point).  Lanes look
// the stencil cells up in parallel; cells whose cluster id cannot improve any
// staged point are skipped.
template <int D, bool F32, bool SPARSE>
__global__ void __launch_bounds__(kCellThreads) k_border_heavy(const gdl::Bufs B, int64_t n) {
  __shared__ DevParams sP;
  __shared__ WarpStage<D> stage[kWarpsPerBlock];
  __shared__ int sIdx[kWarpsPerBlock][32];
  if (threadIdx.x == 0) sP = *B.P;
  __syncthreads();
  const DevParams& P = sP;
  const GridView<SPARSE> gv = view_of<SPARSE>(B);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  WarpStage<D>& S = stage[w];
  const double* __restrict__ X = B.X;
  const float* __restrict__ Xf = B.Xf;
    const int64_t W = (int64_t)gridDim.x * kWarpsPerBlock;
  const OffTab& T = kFullSt[D - 2];
  Tally t;
  const int64_t H = (int64_t)B.ctr[kCtrHeavyBorder];
  for (int64_t h = (int64_t)blockIdx.x * kWarpsPerBlock + w; h < H; h += W) {
    const int64_t m = B.hv_cell[h];
    const int b = B.reps[m], e = B.reps[m + 1];
    const CellXYZ<D> cc = decompose<D>(key_at<SPARSE>(B, b), P);
    for (int c0 = b; c0 < e; c0 += 32) {
      // stage this chunk's non-core points
      const int i = c0 + lane;
      const bool nc = i < e && !B.core[i];
      const unsigned ncm = __ballot_sync(kFull, nc);
      const int na = __popc(ncm);
      if (na == 0) continue;
      if (nc) {
        const int slot = __popc(ncm & ((1u << lane) - 1u));
        sIdx[w][slot] = i;
#pragma unroll
        for (int k = 0; k < D; ++k) {
          S.x[slot][k] = X[k * n + i];
          if (F32) S.f[slot][k] = Xf[k * n + i];
        }
      }
      __syncwarp();
      int best = INT_MAX;  // lane j < na: best cluster of staged point j
      for (int t0 = 0; t0 < T.n; t0 += 32) {
        const int tt = t0 + lane;
        bool has = false;
        int bB = 0, eB = 0, cid = INT_MAX;
        if (tt < T.n) {
          const int64_t kb = offset_key<D>(cc, T.o[tt][0], T.o[tt][1], T.o[tt][2], P);
          if (kb >= 0) {
            const int2 cb = gv.cell((uint64_t)kb);
            bB = cb.x;
            eB = cb.y;
            if (bB < eB && B.cellcore[bB] > 0) {
              has = true;
              cid = B.cellcid[bB];
            }
          }
        }
        unsigned mask = __ballot_sync(kFull, has);
        while (mask) {
          const int src = __ffs(mask) - 1;
          mask &= mask - 1;
          const int cB = __shfl_sync(kFull, cid, src);
          const int cbB = __shfl_sync(kFull, bB, src);
          const int ceB = __shfl_sync(kFull, eB, src);
          unsigned wantm = __ballot_sync(kFull, lane < na && cB < best);
          for (int qb = cbB; qb < ceB && wantm; qb += 32) {
            const int q = qb + lane;
            const bool valid = q < ceB && B.core[q];
            Cand<D, F32> c;
            if (valid) load_cand<D, F32>(c, X, Xf, n, q);
            unsigned pending = wantm;
            while (pending) {
              const int j = __ffs(pending) - 1;
              pending &= pending - 1;
              bool hit = valid && pair_test<D, F32>(S.x[j], S.f[j], c, X, n, q, false, P, t);
              if (__any_sync(kFull, hit)) {
                if (lane == j) best = cB;
                wantm &= ~(1u << j);
              }
            }
          }
        }
      }
      if (lane < na) B.lab[sIdx[w][lane]] = best == INT_MAX ? kNoise : best;
      __syncwarp();
    }
  }
  flush_tally(t, B.ctr);
}

// labels back to the caller's point order; counts
__global__ void k_scatter_labels(const gdl::Bufs B, int64_t n, int* __restrict__ out,
                                 uint8_t* __restrict__ core_out) {
  unsigned long long nn = 0, nc = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t j = B.ids[i];
    const int l = B.lab[i];
    const uint8_t c = B.core[i];
    out[j] = l;
    if (core_out) core_out[j] = c;
    nn += l == kNoise;
    nc += c;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nn += __shfl_xor_sync(kFull, nn, o);
    nc += __shfl_xor_sync(kFull, nc, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (nn) atomicAdd(B.ctr + kCtrNoise, nn);
    if (nc) atomicAdd(B.ctr + kCtrCore, nc);
  }
}

}  // namespace gd

// ------------------------------------------------------------------ launchers
namespace gdl {

using namespace gd;

static int grid_for(int64_t work, int threads, int sms, int per_sm) {
  int64_t g = (work + threads - 1) / threads;
  int64_t cap = (int64_t)sms * per_sm;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

void bbox(const double* pts, int64_t n, int dim, double* partial, int nblocks, int* flags,
          cudaStream_t s) {
  long long* part = reinterpret_cast<long long*>(partial);
  if (dim == 2) k_bbox_partial<2><<<nblocks, kBboxThreads, 0, s>>>(pts, n, part, flags);
  else k_bbox_partial<3><<<nblocks, kBboxThreads, 0, s>>>(pts, n, part, flags);
}

void params(const double* partial, int nblocks, int dim, DevParams* P, double eps, int minpts,
            double cell_mult, uint64_t max_cells, const int* flags, cudaStream_t s) {
  const long long* part = reinterpret_cast<const long long*>(partial);
  if (dim == 2)
    k_params<2><<<1, 256, 0, s>>>(part, nblocks, P, eps, minpts, cell_mult, max_cells, flags);
  else
    k_params<3><<<1, 256, 0, s>>>(part, nblocks, P, eps, minpts, cell_mult, max_cells, flags);
}

void keys(const double* pts, int64_t n, int dim, bool sparse, const DevParams* P, void* keys,
          int sms, cudaStream_t s) {
  int g = grid_for(n, 256, sms, 8);
  using U64 = unsigned long long;
  if (dim == 2) {
    if (sparse) k_keys<2, U64><<<g, 256, 0, s>>>(pts, n, P, static_cast<U64*>(keys));
    else k_keys<2, uint32_t><<<g, 256, 0, s>>>(pts, n, P, static_cast<uint32_t*>(keys));
  } else {
    if (sparse) k_keys<3, U64><<<g, 256, 0, s>>>(pts, n, P, static_cast<U64*>(keys));
    else k_keys<3, uint32_t><<<g, 256, 0, s>>>(pts, n, P, static_cast<uint32_t*>(keys));
  }
}

void gather(const double* pts, const uint32_t* ids, int64_t n, int dim, bool f32,
            const DevParams* P, double* X, float* Xf, int sms, cudaStream_t s) {
  int g = grid_for(n, 256, sms, 8);
  if (dim == 2) {
    if (f32) k_gather<2, true><<<g, 256, 0, s>>>(pts, ids, n, P, X, Xf);
    else k_gather<2, false><<<g, 256, 0, s>>>(pts, ids, n, P, X, Xf);
  } else {
    if (f32) k_gather<3, true><<<g, 256, 0, s>>>(pts, ids, n, P, X, Xf);
    else k_gather<3, false><<<g, 256, 0, s>>>(pts, ids, n, P, X, Xf);
  }
}

void run_flags(const void* keys, bool sparse, int64_t n, uint32_t* fl, int sms, cudaStream_t s) {
  int g = grid_for(n, 256, sms, 8);
  if (sparse)
    k_run_flags<unsigned long long><<<g, 256, 0, s>>>(
        static_cast<const unsigned long long*>(keys), n, fl);
  else
    k_run_flags<uint32_t><<<g, 256, 0, s>>>(static_cast<const uint32_t*>(keys), n, fl);
}

void run_scatter(const uint32_t* fl, const uint32_t* pos, int64_t n, int* reps,
                 const uint32_t* Mdev, unsigned long long* ctr, int sms, cudaStream_t s) {
  k_run_scatter<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(fl, pos, n, reps, Mdev, ctr);
}

void cell_counts(const uint32_t* keys, const int* reps, const uint32_t* Mdev, int64_t n,
                 uint32_t* table, int sms, cudaStream_t s) {
  k_cell_counts<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(keys, reps, Mdev, table);
}

void hash_insert(const unsigned long long* keys, const int* reps, const uint32_t* Mdev, int64_t n,
                 unsigned long long* hkeys, uint32_t* hvals, uint32_t mask, int sms,
                 cudaStream_t s) {
  k_hash_insert<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(keys, reps, Mdev, hkeys, hvals, mask);
}

#define GD_DISPATCH(dim, f32, sparse, KERNEL, GRID, ...)                                    \
  do {                                                                                      \
    if (dim == 2) {                                                                         \
      if (f32) {                                                                            \
        if (sparse) KERNEL<2, true, true><<<GRID, kCellThreads, 0, s>>>(__VA_ARGS__);       \
        else KERNEL<2, true, false><<<GRID, kCellThreads, 0, s>>>(__VA_ARGS__);             \
      } else {                                                                              \
        if (sparse) KERNEL<2, false, true><<<GRID, kCellThreads, 0, s>>>(__VA_ARGS__);      \
        else KERNEL<2, false, false><<<GRID, kCellThreads, 0, s>>>(__VA_ARGS__);            \
      }                                                                                     \
    } else {                                                                                \
      if (f32) {                                                                            \
        if (sparse) KERNEL<3, true, true><<<GRID, kCellThreads, 0, s>>>(__VA_ARGS__);       \
        else KERNEL<3, true, false><<<GRID, kCellThreads, 0, s>>>(__VA_ARGS__);             \
      } else {                                                                              \
        if (sparse) KERNEL<3, false, true><<<GRID, kCellThreads, 0, s>>>(__VA_ARGS__);      \
        else KERNEL<3, false, false><<<GRID, kCellThreads, 0, s>>>(__VA_ARGS__);            \
      }                                                                                     \
    }                                                                                       \
  } while (0)

#define GD_DISPATCH_T(dim, f32, sparse, KERNEL, GRID, THREADS, ...)                         \
  do {                                                                                      \
    if (dim == 2) {                                                                         \
      if (f32) {                                                                            \
        if (sparse) KERNEL<2, true, true><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);            \
        else KERNEL<2, true, false><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);                  \
      } else {                                                                              \
        if (sparse) KERNEL<2, false, true><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);           \
        else KERNEL<2, false, false><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);                 \
      }                                                                                     \
    } else {                                                                                \
      if (f32) {                                                                            \
        if (sparse) KERNEL<3, true, true><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);            \
        else KERNEL<3, true, false><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);                  \
      } else {                                                                              \
        if (sparse) KERNEL<3, false, true><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);           \
        else KERNEL<3, false, false><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);                 \
      }                                                                                     \
    }                                                                                       \
  } while (0)

static int scan_grid(int64_t n, int sms) {
  return grid_for(n, kScanThreadsPerBlock, sms, 8);
}

void core(const Bufs& B, int64_t n, int dim, bool f32, bool sparse, int sms, cudaStream_t s) {
  cudaMemsetAsync(B.ctr + kCtrHeavyCore, 0, 8, s);
  GD_DISPATCH_T(dim, f32, sparse, k_core_scan, scan_grid(n, sms), kScanThreadsPerBlock, B, n);
  GD_DISPATCH(dim, f32, sparse, k_core_heavy, sms * 8, B, n);
}

void unite(const Bufs& B, int64_t n, int dim, bool f32, bool sparse, int sms, cudaStream_t s) {
  k_parent_init<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
  int g = sms * 8;
  for (int pass = 0; pass < 2; ++pass) {
    cudaMemsetAsync(B.ctr + kCtrHeavyUnion, 0, 8, s);
    GD_DISPATCH_T(dim, f32, sparse, k_union_scan, scan_grid(n, sms), kScanThreadsPerBlock, B, n,
                  pass);
    GD_DISPATCH(dim, f32, sparse, k_union_heavy, g, B, n, pass);
  }
  k_compress<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
  k_asym_resolve<<<1, 32, 0, s>>>(B);
}

void roots(const Bufs& B, int64_t n, int sms, cudaStream_t s) {
  k_roots<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
}

void label(const Bufs& B, int64_t n, int sms, cudaStream_t s) {
  k_label<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B, n);
}

void border(const Bufs& B, int64_t n, int dim, bool f32, bool sparse, int sms, cudaStream_t s) {
  cudaMemsetAsync(B.ctr + kCtrHeavyBorder, 0, 8, s);
  GD_DISPATCH_T(dim, f32, sparse, k_border_scan, scan_grid(n, sms), kScanThreadsPerBlock, B, n);
  GD_DISPATCH(dim, f32, sparse, k_border_heavy, sms * 8, B, n);
}

void scatter_labels(const Bufs& B, int64_t n, int* out, uint8_t* core_out, int sms,
                    cudaStream_t s) {
  k_scatter_labels<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B, n, out, core_out);
}

}  // namespace gdl
