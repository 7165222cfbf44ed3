// gd_pipeline.cu -- the exact-DBSCAN kernels.
//
// Replaces, in the reference (CUDA-DClust+):
//   host bbox + bin widths        main.cu:166-207           -> k_bbox_chunk, k_params_inst
//   INDEXING_STRUCTURE/insertData indexing.cu:54-118        -> k_keys (cell keys)
//   thrust::sort_by_key           main.cu:332               -> gdprim::radix_sort_pairs
//   INDEXING_ADJUSTMENT           indexing.cu:23-51         -> k_run_flags/k_run_scatter/
//                                                              k_cell_counts + scan / k_row_hash
//   DBSCAN kernel + searchPoints  dbscan.cu:254-474         -> k_core_point, k_core_heavy
//   MarkAsCandidate + host merge  dbscan.cu:189-222, 25-187 -> k_union_scan, k_union_heavy,
//                                                              k_asym_resolve (device union-find)
//   GetDbscanResult               dbscan.cu:225-251         -> k_roots, k_label, k_border_*,
//                                                              k_scatter_labels
//
// A run clusters K >= 1 independent instances at once: every cell key carries
// the instance id above the instance's local cell key, so one radix sort, one
// cell list and one launch per phase (per dimension present) serve them all.
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
#include <algorithm>
#include <cfloat>
#include <climits>

#include "gd_internal.cuh"
#include "gd_launch.h"

namespace gd {

// ------------------------------------------------------------------ bbox
// Doubles ordered as int64 (monotone for non-NaN values): min/max run on the
// integer pipe instead of the much slower float64 pipe of this GPU.
__device__ __forceinline__ double dbl_of(long long o) {
  return __longlong_as_double(o >= 0 ? o : o ^ 0x7fffffffffffffffLL);
}

__global__ void k_bbox_init(const gdl::Bufs B, int K) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x)
    for (int k = 0; k < 6; ++k) B.bbox[i * 6 + k] = k < 3 ? LLONG_MAX : LLONG_MIN;
}

constexpr int kBboxThreads = 256;

// Calls f(l, x) for every point l in [l0, l1) of an instance whose coordinates
// start at pts (row-major, D doubles per point), x holding its coordinates;
// the block's threads share the range.  With pts 16-byte aligned the points
// come in 16-byte vector loads (2D: one per point, four points in flight per
// thread; 3D: three per pair of points, l0 even), otherwise in scalar loads.
template <int D, class F>
__device__ __forceinline__ void for_points(const double* __restrict__ pts, int64_t l0, int64_t l1,
                                           F&& f) {
  const int t = threadIdx.x, NT = blockDim.x;
  if ((reinterpret_cast<uintptr_t>(pts) & 15) == 0 && (D == 2 || (l0 & 1) == 0)) {
    const double2* __restrict__ p2 = reinterpret_cast<const double2*>(pts);
    if constexpr (D == 2) {
      for (int64_t base = l0; base < l1; base += 4 * NT) {
        double2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int64_t l = base + u * NT + t;
          if (l < l1) v[u] = __ldg(p2 + l);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int64_t l = base + u * NT + t;
          if (l < l1) {
            const double x[3] = {v[u].x, v[u].y, 0.0};
            f(l, x);
          }
        }
      }
    } else {
      const int64_t q0 = l0 >> 1, q1 = l1 >> 1;  // whole pairs: points [2 q0, 2 q1)
      for (int64_t base = q0; base < q1; base += 2 * NT) {
        double2 v[2][3];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int64_t q = base + u * NT + t;
          if (q < q1) {
            v[u][0] = __ldg(p2 + 3 * q);
            v[u][1] = __ldg(p2 + 3 * q + 1);
            v[u][2] = __ldg(p2 + 3 * q + 2);
          }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int64_t q = base + u * NT + t;
          if (q < q1) {
            const double a[3] = {v[u][0].x, v[u][0].y, v[u][1].x};
            f(2 * q, a);
            const double b[3] = {v[u][1].y, v[u][2].x, v[u][2].y};
            f(2 * q + 1, b);
          }
        }
      }
      if ((l1 & 1) && t == 0 && l1 - 1 >= l0) {  // odd last point
        const int64_t l = l1 - 1;
        const double x[3] = {pts[3 * l], pts[3 * l + 1], pts[3 * l + 2]};
        f(l, x);
      }
    }
    return;
  }
  for (int64_t l = l0 + t; l < l1; l += NT) {
    double x[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < D; ++k) x[k] = pts[l * D + k];
    f(l, x);
  }
}

// Order-preserving int64 image of a double's bits (monotone for non-NaN values).
__device__ __forceinline__ long long ord_of(double v) {
  const long long bv = __double_as_longlong(v);
  return bv >= 0 ? bv : bv ^ 0x7fffffffffffffffLL;
}

// one block per chunk of one instance; one atomic per block and bound
__global__ void __launch_bounds__(kBboxThreads) k_bbox_chunk(const gdl::Bufs B) {
  const Chunk c = B.chunks[blockIdx.x];
  const InstDesc I = B.inst[c.inst];
  const int dim = I.dim;
  long long lo[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, hi[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
  bool bad = false;
  const double* __restrict__ pts = B.coords + I.co_off;
  auto take = [&](int64_t, const double* x) {
    for (int k = 0; k < 3; ++k) {
      if (k >= dim) break;
      const long long bv = __double_as_longlong(x[k]);
      bad |= (bv & 0x7ff0000000000000LL) == 0x7ff0000000000000LL;
      const long long o = ord_of(x[k]);
      lo[k] = min(lo[k], o);
      hi[k] = max(hi[k], o);
    }
  };
  if (dim == 2) for_points<2>(pts, c.begin - I.pt_off, c.end - I.pt_off, take);
  else for_points<3>(pts, c.begin - I.pt_off, c.end - I.pt_off, take);
  __shared__ long long s[6][kBboxThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = min(lo[k], __shfl_xor_sync(kFull, lo[k], o));
      hi[k] = max(hi[k], __shfl_xor_sync(kFull, hi[k], o));
    }
    if (lane == 0) { s[k][w] = lo[k]; s[3 + k][w] = hi[k]; }
  }
  if (__any_sync(kFull, bad) && lane == 0) atomicOr(&B.Bi->flags, kFlagNonFinite);
  __syncthreads();
  if (threadIdx.x < 6) {
    const int k = threadIdx.x;
    if ((k % 3) < dim) {
      long long v = s[k][0];
      for (int j = 1; j < kBboxThreads / 32; ++j) v = k < 3 ? min(v, s[k][j]) : max(v, s[k][j]);
      if (k < 3) atomicMin(B.bbox + c.inst * 6 + k, v);
      else atomicMax(B.bbox + c.inst * 6 + k, v);
    }
  }
}

// One thread per instance: its grid and float32 band from its bounding box.
__global__ void k_params_inst(const gdl::Bufs B, int K, double mult2, double mult3,
                              uint64_t dense_floor, uint64_t dense_per_point) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  const InstDesc I = B.inst[i];
  const int D = I.dim;
  const double eps = I.eps;
  DevParams p;
  int fl = 0;
  for (int k = 0; k < 3; ++k) { p.lo[k] = 0; p.hi[k] = 0; p.centre[k] = 0; p.G[k] = 1; }
  if (I.n > 0)
    for (int k = 0; k < D; ++k) {
      p.lo[k] = dbl_of(B.bbox[i * 6 + k]);
      p.hi[k] = dbl_of(B.bbox[i * 6 + 3 + k]);
      p.centre[k] = 0.5 * p.lo[k] + 0.5 * p.hi[k];
    }
  p.dim = D;
  p.minpts = I.minpts;
  p.eps = eps;
  p.eps2 = __dmul_rn(eps, eps);
  p.f = __dmul_rn(eps, D == 2 ? mult2 : mult3);
  p.inv_f = 1.0 / p.f;
  p.pt_off = I.pt_off;
  p.n = I.n;
  p.co_off = I.co_off;
  p.inst = i;
  double cells = 1.0;
  uint64_t C = 1;
  for (int k = 0; k < D; ++k) {
    double t = floor(__dmul_rn(__dsub_rn(p.hi[k], p.lo[k]), p.inv_f)) + 1.0;
    if (!(t < 2147483648.0)) { fl |= kFlagGridTooLarge; t = 1.0; }
    p.G[k] = (int64_t)t;
    cells *= t;
    C *= (uint64_t)p.G[k];
  }
  // local keys must fit 62 bits; a grid beyond the dense-table limit uses the hash
  if (!(cells < 4.0e18)) fl |= kFlagGridTooLarge;
  uint64_t limit = (uint64_t)I.n * dense_per_point;
  if (limit < dense_floor) limit = dense_floor;
  p.C = C;
  p.rows = C / (uint64_t)p.G[D - 1];
  if (!(cells > (double)limit || C > limit)) {
    p.sparse = 0;
  } else {
    // a grid too large for a cell table may still take a table of its rows
    uint64_t rlimit = dense_per_point ? (uint64_t)I.n * kRowsPerPoint : 0;
    if (rlimit < dense_floor) rlimit = dense_floor;
    p.sparse = (fl & kFlagGridTooLarge) || p.rows > rlimit ? 1 : 2;
  }
  udiv_magic((uint64_t)p.G[1], p.dm[0], p.ds[0]);
  udiv_magic((uint64_t)p.G[2], p.dm[1], p.ds[1]);
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
  {
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
    // float64 predicate.  When the bound is not small every pair takes it.
    const double u32 = 1.0 / 16777216.0;               // 2^-24
    R = R * (1.0 + 1e-12) + 1e-300;
    // |fl32(x - c) - (x - c)| and the error of a float32 cell origin (either
    // way of computing it, see cell_origin32), with a small margin
    const double ea = R * u32 * (1.0 + 1.0 / 65536.0);
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
    p.eps2_hi32 = ok ? __double2float_ru(H) : INFINITY;
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
  {
    // float pairs for cell_origin32's float32 path: every cell index below 2^24
    // (exact in float) and magnitudes far from float under- and overflow
    bool fast = p.f >= 0x1p-60 && p.f <= 0x1p60;
    p.f_hi = __double2float_rn(p.f);
    p.f_lo = __double2float_rn(p.f - (double)p.f_hi);
    for (int k = 0; k < 3; ++k) {
      const double b = k < D ? p.lo[k] - p.centre[k] : 0.0;
      fast = fast && p.G[k] < (1 << 24) && fabs(b) <= 0x1p60;
      p.b_hi[k] = __double2float_rn(b);
      p.b_lo[k] = __double2float_rn(b - (double)p.b_hi[k]);
    }
    p.fast_origin = fast ? 1 : 0;
  }
  {
    // Float32 cell keys.  k_keys computes t64 = fl64(fl64(x - lo) * inv_f) and
    // floor(t64).  Its float32 path takes x32 = x rounded toward zero (from the
    // bits, |x32 - x| <= |x| 2^-23), lo32 = fl32(lo), i32 = fl32(inv_f) and
    // t32 = fl32(fl32(x32 - lo32) * i32).  With T = (x - lo) inv_f exact,
    //   |t32 - T| <= (|x| 2^-23 + |lo| 2^-24) inv_f (1 + 2^-22) + T (3 2^-24 + 2^-47)
    //   |t64 - T| <= T 2^-52,
    // and 0 <= T <= (hi - lo) inv_f < G + 1.  key_band is 1.25 times the sum
    // (rounded up to float): a t32 farther than that from every integer has
    // floor(t32) = floor(t64).
    double maxabs_k = 0.0, loabs = 0.0;
    for (int k = 0; k < D; ++k) {
      maxabs_k = fmax(maxabs_k, fmax(fabs(p.lo[k]), fabs(p.hi[k])));
      loabs = fmax(loabs, fabs(p.lo[k]));
    }
    double gmax = 1.0;
    for (int k = 0; k < D; ++k) gmax = fmax(gmax, (double)p.G[k]);
    const double band = 1.25 * ((maxabs_k * 0x1p-23 + loabs * 0x1p-24) * p.inv_f * (1.0 + 0x1p-22) +
                                (gmax + 1.0) * (3.0 * 0x1p-24 + 0x1p-47));
    bool kf = I.n > 0 && band < 0.125 && gmax < 0x1p21 && maxabs_k < 0x1p100 && p.inv_f < 0x1p100 &&
              maxabs_k * p.inv_f < 0x1p100;
    for (int k = 0; k < 3; ++k) p.key_lo32[k] = k < D ? __double2float_rn(p.lo[k]) : 0.0f;
    p.key_inv32 = __double2float_rn(p.inv_f);
    p.key_band = __double2float_ru(band);
    p.key_fast = kf ? 1 : 0;
  }
  p.flags = fl;
  p.occ_off = 0;
  p.start_off = 0;
  p.m0 = 0;
  p.m1 = -1;
  p.rank_off = 0;
  p.kmask = 0;
  p.LB = 0;
  B.Pv[i] = p;
}

// One block: the run layout -- key widths, cell-table offsets (exclusive scan
// over every instance's table length), flags.
__global__ void __launch_bounds__(1024) k_layout(const gdl::Bufs B, int K) {
  __shared__ unsigned long long s_part[32], s_part2[32];
  __shared__ int s_red[4][32];
  __shared__ unsigned long long s_carry, s_carry2;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int lb = 0, fl = 0, sp = 0, xf = 0, md = 2, k2 = 0;
  for (int i = threadIdx.x; i < K; i += blockDim.x) {
    const DevParams& p = B.Pv[i];
    if (p.n > 0) lb = max(lb, p.key_bits);
    fl |= p.flags;
    sp |= p.sparse == 1;
    xf |= p.prune;
    if (p.n > 0 && !(p.eps2_lo32 > 0.0f)) xf |= 2;
    md = max(md, p.dim);
    k2 += p.dim == 2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lb = max(lb, __shfl_xor_sync(kFull, lb, o));
    fl |= __shfl_xor_sync(kFull, fl, o);
    sp |= __shfl_xor_sync(kFull, sp, o);
    xf |= __shfl_xor_sync(kFull, xf, o);
    md = max(md, __shfl_xor_sync(kFull, md, o));
    k2 += __shfl_xor_sync(kFull, k2, o);
  }
  if (lane == 0) {
    s_red[0][w] = lb;
    s_red[1][w] = fl | (sp << 16) | (xf << 17);
    s_red[2][w] = md;
    s_red[3][w] = k2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int LB = 0, F = 0, MD = 2, K2 = 0;
    for (int j = 0; j < 32; ++j) {
      LB = max(LB, s_red[0][j]);
      F |= s_red[1][j];
      MD = max(MD, s_red[2][j]);
      K2 += s_red[3][j];
    }
    int IB = 0;
    while (IB < 31 && ((K - 1) >> IB)) ++IB;
    BatchInfo bi;
    bi.K = K;
    bi.LB = LB;
    bi.IB = IB;
    bi.key64 = LB + IB > 32 ? 1 : 0;
    bi.any_sparse = (F >> 16) & 1;
    bi.any_xf = (F >> 17) & 1;
    bi.flags = (F & 0xffff) | B.Bi->flags | (LB + IB > 62 ? kFlagGridTooLarge : 0);
    bi.max_dim = MD;
    bi.K2 = K2;
    bi.band_off = (F >> 18) & 1;
    bi.occ_total = 0;
    bi.start_total = 0;
    *B.Bi = bi;
    s_carry = 0;
    s_carry2 = 0;
  }
  __syncthreads();
  const int LB = B.Bi->LB;
  const uint64_t kmask = LB >= 64 ? ~0ull : ((1ull << LB) - 1ull);
  // exclusive scans of the table sizes, 1024 instances at a time: occupancy
  // bits (C+1 per cell table, rows+1 per row table, none for the hash) and
  // start entries (rows+1 per row table, else one entry holding the point
  // count, so the start scan stays in sorted-position units)
  for (int base = 0; base < K; base += 1024) {
    const int i = base + threadIdx.x;
    unsigned long long vo = 0, vs = 0;
    if (i < K) {
      const DevParams& p = B.Pv[i];
      vo = p.sparse == 1 ? 0 : (p.sparse == 2 ? p.rows : p.C) + 1;
      vs = p.sparse == 2 ? p.rows + 1 : 1;
    }
    unsigned long long io = vo, is = vs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long t = __shfl_up_sync(kFull, io, o), u = __shfl_up_sync(kFull, is, o);
      if (lane >= o) {
        io += t;
        is += u;
      }
    }
    if (lane == 31) {
      s_part[w] = io;
      s_part2[w] = is;
    }
    __syncthreads();
    if (w == 0) {
      const unsigned long long t = s_part[lane], u = s_part2[lane];
      unsigned long long ti = t, ui = u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long a = __shfl_up_sync(kFull, ti, o), c = __shfl_up_sync(kFull, ui, o);
        if (lane >= o) {
          ti += a;
          ui += c;
        }
      }
      s_part[lane] = ti - t;
      s_part2[lane] = ui - u;
    }
    __syncthreads();
    const unsigned long long eo = s_carry + s_part[w] + io - vo;
    const unsigned long long es = s_carry2 + s_part2[w] + is - vs;
    if (i < K) {
      B.Pv[i].occ_off = eo;
      B.Pv[i].start_off = es;
      B.Pv[i].kmask = kmask;
      B.Pv[i].LB = LB;
    }
    __syncthreads();
    if (threadIdx.x == 1023) {
      s_carry = eo + vo;
      s_carry2 = es + vs;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    B.Bi->occ_total = s_carry;
    B.Bi->start_total = s_carry2;
  }
}

// ------------------------------------------------------------------ keys
// floor(fl64(fl64(x - lo) * inv_f)) as an int: t is finite; out-of-range
// values saturate, and the caller's clamp takes them to the grid's edge.
__device__ __forceinline__ int cell_index_f64(double x, double lo, double inv_f) {
  return __double2int_rd(__dmul_rn(__dsub_rn(x, lo), inv_f));
}

// One block per chunk: cell key of every point, instance id above the local key.
template <class Key>
__global__ void __launch_bounds__(256) k_keys(const gdl::Bufs B, Key* __restrict__ keys) {
  const Chunk c = B.chunks[blockIdx.x];
  const DevParams& P = B.Pv[c.inst];
  const int D = P.dim;
  double lo[3], inv_f = P.inv_f;
  int64_t G[3];
  for (int k = 0; k < 3; ++k) { lo[k] = P.lo[k]; G[k] = P.G[k]; }
  const uint64_t hi = (uint64_t)P.inst << P.LB;
  const bool kfast = P.key_fast != 0;
  const float band = P.key_band, inv32 = P.key_inv32;
  float lo32[3];
  for (int k = 0; k < 3; ++k) lo32[k] = P.key_lo32[k];
  const double* __restrict__ pts = B.coords + P.co_off;
  Key* __restrict__ out = keys + P.pt_off;
  auto key_of = [&](int64_t l, const double* xs) {
    uint64_t key = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (k >= D) break;
      const double x = xs[k];
      // 32-bit cell index: conversions to 64-bit integers run on this GPU's
      // narrow float64 pipe; every cell index is below 2^31 (grids are checked)
      int q;
      bool fast = false;
      if (kfast) {
        // float32 cell position (no float64 instruction), used when it is
        // farther than key_band from a cell boundary
        const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
        const int fe = (int)((bits >> 52) & 0x7ff) - 1023 + 127;
        const bool zero = (bits << 1) == 0;
        if (zero || (fe > 0 && fe < 255)) {
          const unsigned sgn = (unsigned)(bits >> 63) << 31;
          const float x32 = zero ? 0.0f
                                 : __uint_as_float(sgn | ((unsigned)fe << 23) |
                                                   (unsigned)((bits >> 29) & 0x7fffffu));
          const float t = __fmul_rn(__fsub_rn(x32, lo32[k]), inv32);
          if (fabsf(t) < 4194304.0f) {
            // floor without a conversion instruction: for |t| < 2^22,
            // t + 1.5 * 2^23 rounded down lies in [2^23, 2^24), where floats are
            // the integers, so it is floor(t) + 1.5 * 2^23 exactly and its
            // mantissa bits hold floor(t) + 2^22
            const float s = __fadd_rd(t, 12582912.0f);
            const float fl = __fsub_rn(s, 12582912.0f);
            const float fr = __fsub_rn(t, fl);
            if (fr > band && fr < 1.0f - band) {
              q = (int)(__float_as_uint(s) - 0x4b400000u);
              fast = true;
            }
          }
        }
      }
      // the float64 formula for the few coordinates near a cell boundary
      if (!fast) q = cell_index_f64(x, lo[k], inv_f);
      q = q < 0 ? 0 : ((int64_t)q >= G[k] ? (int)(G[k] - 1) : q);
      key = key * (uint64_t)G[k] + (uint64_t)q;
    }
    out[l] = (Key)(hi | key);
  };
  if (D == 2) for_points<2>(pts, c.begin - P.pt_off, c.end - P.pt_off, key_of);
  else for_points<3>(pts, c.begin - P.pt_off, c.end - P.pt_off, key_of);
}

template <class Key>
__device__ __forceinline__ int inst_of(Key key, int LB) {
  return (int)((uint64_t)key >> LB);
}

// Coordinates of one point in 16-byte loads where the address allows (a 2D
// point at a 16-byte boundary is one load; a 3D point is a 16-byte and an
// 8-byte load, in the order its alignment allows).
template <int D>
__device__ __forceinline__ void load_coords(const double* __restrict__ src, double* v) {
  const bool a16 = (reinterpret_cast<uintptr_t>(src) & 15) == 0;
  if (D == 2) {
    if (a16) {
      const double2 t = __ldg(reinterpret_cast<const double2*>(src));
      v[0] = t.x;
      v[1] = t.y;
    } else {
      v[0] = __ldg(src);
      v[1] = __ldg(src + 1);
    }
  } else {
    if (a16) {
      const double2 t = __ldg(reinterpret_cast<const double2*>(src));
      v[0] = t.x;
      v[1] = t.y;
      v[2] = __ldg(src + 2);
    } else {
      v[0] = __ldg(src);
      const double2 t = __ldg(reinterpret_cast<const double2*>(src + 1));
      v[1] = t.x;
      v[2] = t.y;
    }
  }
}

// Sorted structure-of-arrays copy (+ centred float32 copy).  ONE: a single
// instance (its parameters are Pv[0], no key is read).  kGatherU points per
// thread and pass, so that as many random loads are in flight.
#ifndef GD_GATHER_U
#define GD_GATHER_U 4
#endif
constexpr int kGatherU = GD_GATHER_U;
template <class Key, bool XF, bool ONE>
__global__ void k_gather(const gdl::Bufs B, int64_t n) {
  const int LB = B.Bi->LB;
  const Key* __restrict__ keys = static_cast<const Key*>(B.keys);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += kGatherU * stride) {
    double v[kGatherU][3];
    const DevParams* Pp[kGatherU];
#pragma unroll
    for (int u = 0; u < kGatherU; ++u) {
      const int64_t i = i0 + u * stride;
      Pp[u] = nullptr;
      if (i < n) {
        const int64_t g = B.ids[i];
        const DevParams& P = B.Pv[ONE ? 0 : inst_of(keys[i], LB)];
        Pp[u] = &P;
        const double* src = B.coords + P.co_off + (g - P.pt_off) * P.dim;
        if (P.dim == 2) load_coords<2>(src, v[u]);
        else load_coords<3>(src, v[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < kGatherU; ++u) {
      const int64_t i = i0 + u * stride;
      if (i >= n) continue;
      const DevParams& P = *Pp[u];
      const int D = P.dim;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k >= D) break;
        B.X[k * n + i] = v[u][k];
        if (XF) B.Xf[k * n + i] = __double2float_rn(__dsub_rn(v[u][k], P.centre[k]));
      }
    }
  }
}

// ---------------------------------------------------------------- bit masks
// Number of set bits of a mask below position i (0 <= i <= its length): the
// word prefix count plus the set bits of i's word below it.
__device__ __forceinline__ uint32_t bit_rank(const uint32_t* __restrict__ bits,
                                             const uint32_t* __restrict__ pre, int64_t i) {
  const int64_t w = i >> 5;
  return pre[w] + (uint32_t)__popc(bits[w] & ((1u << (i & 31)) - 1u));
}

// Cell index m of sorted position i: the cell starts at or before i, less one.
__device__ __forceinline__ int cell_of(const gdl::Bufs& B, int64_t i) {
  const int64_t w = i >> 5;
  return (int)(B.runpre[w] + (uint32_t)__popc(B.runbits[w] & (0xffffffffu >> (31 - (i & 31))))) -
         1;
}

// Cell starts: one bit per sorted position (a key differing from the one
// before it), written a word per warp.
template <class Key>
__global__ void k_run_bits(const Key* __restrict__ keys, int64_t n, uint32_t* __restrict__ bits) {
  const int lane = threadIdx.x & 31;
  // four groups of 32 positions per warp and pass, their loads issued together
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t g0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); g0 < n;
       g0 += U * stride) {
    Key k[U], p[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = g0 + u * stride + lane;
      k[u] = i < n ? keys[i] : (Key)0;
      p[u] = lane == 0 && i > 0 && i <= n ? keys[i - 1] : (Key)0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i0 = g0 + u * stride;
      if (i0 >= n) break;  // warp-uniform
      const int64_t i = i0 + lane;
      Key prev = __shfl_up_sync(kFull, k[u], 1);
      if (lane == 0) prev = p[u];
      const unsigned b = __ballot_sync(kFull, i < n && (i == 0 || k[u] != prev));
      if (lane == 0) bits[i0 >> 5] = b;
    }
  }
}

// After the cell starts are listed in reps: reps[M] = n, the cell count, and
// (mixed runs) the number of cells of 2D instances -- 2D instances come first,
// the first cell of a 3D instance is found by binary search.
template <class Key>
__global__ void k_runs_finish(const gdl::Bufs B, int64_t n, int mixed) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int64_t M = *B.M;
  B.reps[M] = (int)n;
  B.ctr[kCtrCells] = (unsigned long long)M;
  const int K2 = B.Bi->K2;
  int64_t lo = K2 > 0 ? M : 0;
  if (mixed) {
    const Key* keys = static_cast<const Key*>(B.keys);
    const int LB = B.Bi->LB;
    int64_t hi = M;  // first cell with instance >= K2
    lo = 0;
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if (inst_of(keys[B.reps[mid]], LB) < K2) lo = mid + 1;
      else hi = mid;
    }
  }
  B.ctr[kCtrCells2D] = (unsigned long long)lo;
}

// Cell tables: one occupancy bit per non-empty cell (a cell's points are then
// found by rank, see GridView::rank).  Row tables: one occupancy bit and a cell
// count per non-empty row (scanned afterwards into each row's first cell).
// Every cell's last-axis coordinate goes to cellz, and each instance's first
// and last cells are recorded (k_start_fill turns them into the one-entry start
// slices of the other instances, so the scan stays in cell units).
template <class Key>
__global__ void k_cell_counts(const gdl::Bufs B) {
  const Key* keys = static_cast<const Key*>(B.keys);
  const int LB = B.Bi->LB;
  const int64_t M = *B.M;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    const Key key = keys[B.reps[m]];
    const int inst = inst_of(key, LB);
    DevParams& P = B.Pv[inst];
    if (m == 0 || inst_of(keys[B.reps[m - 1]], LB) != inst) P.m0 = m;
    if (m == M - 1 || inst_of(keys[B.reps[m + 1]], LB) != inst) P.m1 = m;
    const uint64_t local = (uint64_t)key & P.kmask;
    const int a = P.dim - 2;
    const uint64_t row = udiv_by(local, P.dm[a], P.ds[a]);
    B.cellz[m] = (uint32_t)(local - row * (uint64_t)P.G[P.dim - 1]);
    if (P.sparse == 1) continue;
    if (P.sparse == 2) {
      atomicAdd(B.start + P.start_off + row, 1u);
      const uint64_t idx = P.occ_off + row;
      atomicOr(B.occ + (idx >> 5), 1u << (idx & 31));
      continue;
    }
    const uint64_t idx = P.occ_off + local;
    atomicOr(B.occ + (idx >> 5), 1u << (idx & 31));
  }
}

// One-entry start slices (instances without a row table): their cell count.
__global__ void k_start_fill(const gdl::Bufs B, int K) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
    const DevParams& P = B.Pv[i];
    if (P.sparse != 2) B.start[P.start_off] = P.n > 0 ? (uint32_t)(P.m1 - P.m0 + 1) : 0u;
  }
}

// A cell table's cells appear in reps in table order from the instance's first
// cell on, so a cell's index into reps is its occupancy rank minus the rank of
// the table's first bit plus that first cell.
__global__ void k_rank_off(const gdl::Bufs B, int K) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
    DevParams& P = B.Pv[i];
    if (P.sparse != 0 || P.n == 0) continue;
    const uint64_t idx = P.occ_off, w = idx >> 5;
    const int64_t r = (int64_t)B.wpre[w] + __popc(B.occ[w] & ((1u << (idx & 31)) - 1u));
    P.rank_off = P.m0 - r;
  }
}

// sparse instances: hash of the occupied rows, global key of the row's first
// cell -> [begin, end) of the row's points.  The thread of a row's first cell
// walks the row's cells to its end.
template <class Key>
__global__ void k_row_hash(const gdl::Bufs B) {
  const Key* keys = static_cast<const Key*>(B.keys);
  const int LB = B.Bi->LB;
  const int64_t M = *B.M;
  const uint32_t mask = B.hmask;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t key = (uint64_t)keys[B.reps[m]];
    const int inst = (int)(key >> LB);
    const DevParams& P = B.Pv[inst];
    if (P.sparse != 1) continue;
    const uint64_t Gl = (uint64_t)P.G[P.dim - 1];
    const uint64_t hi = key & ~P.kmask;
    const uint64_t local = key & P.kmask;
    const uint64_t rowkey = local - local % Gl;
    if (m > 0) {
      const uint64_t pk = (uint64_t)keys[B.reps[m - 1]];
      if ((pk & ~P.kmask) == hi && (pk & P.kmask) >= rowkey) continue;  // not the row's first cell
    }
    int64_t m2 = m + 1;
    while (m2 < M) {
      const uint64_t k2 = (uint64_t)keys[B.reps[m2]];
      if ((k2 & ~P.kmask) != hi || (k2 & P.kmask) >= rowkey + Gl) break;
      ++m2;
    }
    const unsigned long long k = hi | rowkey;
    uint32_t h = hash_key(k) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
      unsigned long long prev = atomicCAS(B.hkeys + h, kHashEmpty, k);
      if (prev == kHashEmpty || prev == k) {
        B.hvals[2 * h] = (uint32_t)B.reps[m];
        B.hvals[2 * h + 1] = (uint32_t)B.reps[m2];
        break;
      }
      h = (h + 1) & mask;
    }
  }
}

// ------------------------------------------------------------- cell helpers
template <int D>
struct CellXYZ {
  int c[3];  // per-axis cell indices (each below 2^31)
};

template <int D>
__device__ __forceinline__ CellXYZ<D> decompose(uint64_t key, const DevParams& P) {
  CellXYZ<D> r;
  uint64_t k = key;
  if (D == 3) {
    const uint64_t k2 = udiv_by(k, P.dm[1], P.ds[1]);
    r.c[2] = (int)(k - k2 * (uint64_t)P.G[2]);
    k = k2;
  } else {
    r.c[2] = 0;
  }
  const uint64_t k1 = udiv_by(k, P.dm[0], P.ds[0]);
  r.c[1] = (int)(k - k1 * (uint64_t)P.G[1]);
  r.c[0] = (int)k1;
  return r;
}

// key of cell (c + o), or -1 when outside the grid
template <int D>
__device__ __forceinline__ int64_t offset_key(const CellXYZ<D>& c, int ox, int oy, int oz,
                                              const DevParams& P) {
  int64_t x = (int64_t)c.c[0] + ox, y = (int64_t)c.c[1] + oy;
  if (x < 0 || x >= P.G[0] || y < 0 || y >= P.G[1]) return -1;
  int64_t k = x * P.G[1] + y;
  if (D == 3) {
    int64_t z = (int64_t)c.c[2] + oz;
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
// (sorted position si; float64 coordinates sx in float64 mode), the other a
// candidate (sorted position q; coordinates in registers).  stage_is_centre
// selects which is the centre of the query box.  In float32-band mode the
// float64 coordinates of both are loaded only for a band re-test.
template <int D, bool F32, class PP>
__device__ __forceinline__ bool pair_test(const double* sx, const float* sf, const Cand<D, F32>& c,
                                          const double* __restrict__ X, int64_t n, int64_t q,
                                          int64_t si, bool stage_is_centre, const PP& P,
                                          Tally& t) {
  if (F32) {
    ++t.t32;
    float s = dist2_f32<D>(sf, c.f);
    if (s < P.eps2_lo32) return true;
    if (s > P.eps2_hi32) return false;
    ++t.band;
    double qx[D], px[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      qx[k] = X[k * n + q];
      px[k] = X[k * n + si];
    }
    ++t.t64;
    double d2 = dist2_f64<D>(px, qx);
    return stage_is_centre ? pred_from_d2<D>(d2, px, qx, P) : pred_from_d2<D>(d2, qx, px, P);
  } else {
    ++t.t64;
    double d2 = dist2_f64<D>(sx, c.x);
    return stage_is_centre ? pred_from_d2<D>(d2, sx, c.x, P) : pred_from_d2<D>(d2, c.x, sx, P);
  }
}

// Symmetric test for core-core links: true when the pair is a neighbour in both
// directions; counts pairs that are neighbours in exactly one direction.
template <int D, bool F32, class PP>
__device__ __forceinline__ bool link_test(const double* sx, const float* sf, const Cand<D, F32>& c,
                                          const double* __restrict__ X, int64_t n, int a, int q,
                                          const PP& P, Tally& t,
                                          int* __restrict__ asym_list, unsigned long long* ctr) {
  double qx[D], ax[D];
  if (F32) {
    ++t.t32;
    float s = dist2_f32<D>(sf, c.f);
    if (s < P.eps2_lo32) return true;
    if (s > P.eps2_hi32) return false;
    ++t.band;
    // float64 coordinates of both, for the band re-test only
#pragma unroll
    for (int k = 0; k < D; ++k) {
      qx[k] = X[k * n + q];
      ax[k] = X[k * n + a];
    }
  } else {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      qx[k] = c.x[k];
      ax[k] = sx[k];
    }
  }
  sx = ax;
  ++t.t64;
  double d2 = dist2_f64<D>(sx, qx);
  if (d2_le(d2, P.eps2_in)) return true;
  if (!d2_le(d2, P.eps2)) return false;
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

// The lanes sharing this lane's value v, for values that sit in runs of
// consecutive lanes (lanes holding sorted points: a cell's points are
// neighbours).  act: the lanes taking part; the result is the run of
// consecutive active lanes with v that holds this lane (0 for an inactive
// lane).  Equal values split by an inactive lane give two runs.  All 32 lanes
// call it.  (__match_any_sync gives the same sets for such values, at a
// higher cost.)
__device__ __forceinline__ unsigned run_peers(unsigned act, int v) {
  const int lane = threadIdx.x & 31;
  const int prev = __shfl_up_sync(kFull, v, 1);
  const bool on = (act >> lane) & 1u;
  const bool prev_on = ((act << 1) >> lane) & 1u;             // lane - 1 active (0 for lane 0)
  const bool head = on && (!prev_on || prev != v);
  const unsigned heads = __ballot_sync(kFull, head);
  if (!on) return 0u;
  const unsigned upto = (unsigned)((2ull << lane) - 1ull);   // lanes 0..lane
  const int s = 31 - __clz(heads & upto);                     // this run's head
  const unsigned stop = (heads | ~act) & ~upto;               // next head or gap
  const int e = stop ? __ffs(stop) - 1 : 32;
  return (unsigned)(((1ull << e) - 1ull) & ~((1ull << s) - 1ull));
}

// Cell lookup inside one instance.  Dense grids: the instance's slice of the
// cell tables gives every cell's point range (an occupancy bit per entry skips
// empty cells without touching the table).  Sparse grids: a hash of the
// occupied rows (all cells sharing every coordinate but the last) gives the
// row's point range, and a binary search on the sorted keys the cells inside
// it.  The probe loop is bounded by the table size.  The view holds only the
// instance's scalars; the tables' addresses are read from the kernel's
// parameter block at each use (B is always the kernel parameter), so they
// occupy no registers in the walks.
struct GridView {
  int sparse;              // DevParams::sparse
  int key64;
  uint64_t occ_off;
  uint64_t start_off;
  int64_t rank_off;
  uint64_t hi;             // instance id << LB
  int64_t Gl;              // cells along the last axis
  uint64_t glm;            // division by Gl (udiv_by)
  int32_t gls;

  __device__ __forceinline__ uint64_t gkey(const gdl::Bufs& B, int64_t i) const {
    return key64 ? static_cast<const unsigned long long*>(B.keys)[i]
                 : (uint64_t) static_cast<const uint32_t*>(B.keys)[i];
  }
  // cell table: index into reps of the first non-empty cell at or after
  // local key k (its rank among the occupied cells)
  __device__ __forceinline__ int64_t rank(const gdl::Bufs& B, uint64_t k) const {
    const uint64_t idx = occ_off + k, w = idx >> 5;
    return (int64_t)B.wpre[w] + __popc(B.occ[w] & ((1u << (idx & 31)) - 1u)) + rank_off;
  }
  __device__ __forceinline__ bool occupied(const gdl::Bufs& B, uint64_t k) const {
    const uint64_t idx = occ_off + k;
    return (B.occ[idx >> 5] >> (idx & 31)) & 1u;
  }
  // row table: cells [begin, end) (indices into reps) of row ri
  __device__ __forceinline__ int2 row_cells(const gdl::Bufs& B, uint64_t ri) const {
    const uint64_t idx = occ_off + ri;
    if (!((B.occ[idx >> 5] >> (idx & 31)) & 1u)) return make_int2(0, 0);
    return make_int2((int)B.start[start_off + ri], (int)B.start[start_off + ri + 1]);
  }
  // first cell in [b, e) (one row's cells) whose last-axis coordinate is >= z
  __device__ __forceinline__ int zlower(const gdl::Bufs& B, int b, int e, int64_t z) const {
    while (b < e) {
      const int mid = (int)(((unsigned)b + (unsigned)e) >> 1);
      if ((int64_t)B.cellz[mid] < z) b = mid + 1;
      else e = mid;
    }
    return b;
  }
  // row table: whether row ri holds a core point
  __device__ __forceinline__ bool core_row_at(const gdl::Bufs& B, uint64_t ri) const {
    const uint64_t idx = occ_off + ri;
    return (B.cocc[idx >> 5] >> (idx & 31)) & 1u;
  }
  // hash: points [begin, end) of the row whose first cell is rowkey
  __device__ __forceinline__ int2 row(const gdl::Bufs& B, uint64_t rowkey) const {
    const unsigned long long k = hi | rowkey;
    const uint32_t hmask = B.hmask;
    uint32_t h = hash_key(k) & hmask;
    for (uint32_t probe = 0; probe <= hmask; ++probe) {
      const unsigned long long kk = B.hkeys[h];
      if (kk == k) return make_int2((int)B.hvals[2 * h], (int)B.hvals[2 * h + 1]);
      if (kk == kHashEmpty) break;
      h = (h + 1) & hmask;
    }
    return make_int2(0, 0);
  }
  // cell table: occupancy bits of cells z0..z1 (at most 5) of the row whose
  // first cell is rowkey (bit z - z0), and the reps index of the first
  // occupied one (the others follow it in reps).  The three words are loaded
  // at once, whether or not they are needed: word w + 1 past the last
  // occupancy word is the first core occupancy word, in the same buffer.
  __device__ __forceinline__ uint32_t occ_cells(const gdl::Bufs& B, uint64_t rowkey, int64_t z0,
                                                int64_t z1, int64_t& r0) const {
    const uint64_t i0 = occ_off + rowkey + (uint64_t)z0, w = i0 >> 5;
    const int len = (int)(z1 - z0) + 1;
    const int sh = (int)(i0 & 31);
    const uint32_t lo = B.occ[w], hi = B.occ[w + 1], pre = B.wpre[w];
    const uint64_t bits = (((uint64_t)hi << 32) | lo) >> sh;
    const uint32_t mask = (uint32_t)bits & ((1u << len) - 1u);
    r0 = (int64_t)pre + __popc(lo & ((1u << sh) - 1u)) + rank_off;
    return mask;
  }
  // core occupancy bits of cells z0..z1 of a cell-table row (bit z - z0); word
  // w + 1 past the last one lies in the padding or the word prefix counts
  // that follow in the same buffer
  __device__ __forceinline__ uint32_t core_cells(const gdl::Bufs& B, uint64_t rowkey, int64_t z0,
                                                 int64_t z1) const {
    const uint64_t i0 = occ_off + rowkey + (uint64_t)z0;
    const int len = (int)(z1 - z0) + 1;  // <= 5
    const uint64_t w = i0 >> 5;
    const int sh = (int)(i0 & 31);
    const uint64_t bits = (((uint64_t)B.cocc[w + 1] << 32) | B.cocc[w]) >> sh;
    return (uint32_t)bits & ((1u << len) - 1u);
  }
  // first sorted position in [b, e) whose key is >= g
  __device__ __forceinline__ int lower(const gdl::Bufs& B, int b, int e, uint64_t g) const {
    while (b < e) {
      const int mid = (int)(((unsigned)b + (unsigned)e) >> 1);
      if (gkey(B, mid) < g) b = mid + 1;
      else e = mid;
    }
    return b;
  }
  // points of the cells z0..z1 of the row whose first cell is rowkey: one
  // contiguous range, because no other key sorts between them
  __device__ __forceinline__ int2 span_row(const gdl::Bufs& B, uint64_t rowkey, int64_t z0,
                                           int64_t z1) const {
    if (!sparse)
      return make_int2(B.reps[rank(B, rowkey + z0)], B.reps[rank(B, rowkey + z1 + 1)]);
    if (sparse == 2) {
      const int2 rc = row_cells(B, udiv_by(rowkey, glm, gls));
      if (rc.x == rc.y) return make_int2(0, 0);
      const int ma = zlower(B, rc.x, rc.y, z0), mb = zlower(B, ma, rc.y, z1 + 1);
      return make_int2(B.reps[ma], B.reps[mb]);
    }
    const int2 r = row(B, rowkey);
    if (r.x == r.y) return r;
    const int a = lower(B, r.x, r.y, hi | (rowkey + (uint64_t)z0));
    const int b = lower(B, a, r.y, hi | (rowkey + (uint64_t)z1 + 1));
    return make_int2(a, b);
  }
  // points of the cell with local key k: [x, y)
  __device__ __forceinline__ int2 cell(const gdl::Bufs& B, uint64_t k) const {
    if (!sparse) {
      if (!occupied(B, k)) return make_int2(0, 0);
      const int64_t r = rank(B, k);
      return make_int2(B.reps[r], B.reps[r + 1]);
    }
    const int64_t z = (int64_t)(k - udiv_by(k, glm, gls) * (uint64_t)Gl);
    return span_row(B, k - (uint64_t)z, z, z);
  }
  // points of the cells k0..k1 (consecutive local keys along one row)
  __device__ __forceinline__ int2 span(const gdl::Bufs& B, uint64_t k0, uint64_t k1) const {
    if (!sparse) return make_int2(B.reps[rank(B, k0)], B.reps[rank(B, k1 + 1)]);
    const int64_t z0 = (int64_t)(k0 - udiv_by(k0, glm, gls) * (uint64_t)Gl);
    return span_row(B, k0 - (uint64_t)z0, z0, z0 + (int64_t)(k1 - k0));
  }
};

__device__ __forceinline__ GridView view_of(const gdl::Bufs& B, const DevParams& P) {
  const int a = P.dim - 2;
  return GridView{P.sparse, B.Bi->key64, P.occ_off, P.start_off, P.rank_off,
                  (uint64_t)P.inst << P.LB, P.G[P.dim - 1], P.dm[a], P.ds[a]};
}

template <bool KEY64>
__device__ __forceinline__ uint64_t key_at(const gdl::Bufs& B, int64_t i) {
  if (KEY64) return static_cast<const unsigned long long*>(B.keys)[i];
  return static_cast<const uint32_t*>(B.keys)[i];
}

// The cell a kernel thread/warp works on: instance parameters and local key.
struct CellCtx {
  const DevParams* P;
  uint64_t local;
};

template <bool KEY64>
__device__ __forceinline__ CellCtx cell_ctx(const gdl::Bufs& B, int b, int LB) {
  const uint64_t key = key_at<KEY64>(B, b);
  CellCtx c;
  c.P = B.Pv + (int)(key >> LB);
  c.local = key & c.P->kmask;
  return c;
}

// cell range of dimension D: 2D instances' cells come first
template <int D>
__device__ __forceinline__ void dim_range(const gdl::Bufs& B, int64_t& mlo, int64_t& mhi) {
  const int64_t M = *B.M, M2 = (int64_t)B.ctr[kCtrCells2D];
  mlo = D == 2 ? 0 : M2;
  mhi = D == 2 ? M2 : M;
}

// ------------------------------------------------------------ stencil tables
// Offsets within +-2 cells, built at compile time.  kRows: the (ox, oy) rows a
// core count scans, nearest first (by the smallest possible distance to the
// row, then by how many axes are off), so that points in dense regions reach
// minPts in fewer rows.  kHalf[d][pass]: the half stencil (o > 0
// lexicographically) split into the union passes (union_pass).  kFullSt[d]:
// all offsets (the warp border search).
struct OffTab {
  signed char o[128][3];
  int n;
};

constexpr int row_rank(int x, int y) {
  const int ax = x < 0 ? -x : x, ay = y < 0 ? -y : y;
  const int gx = ax > 1 ? ax - 1 : 0, gy = ay > 1 ? ay - 1 : 0;  // empty cells between
  return (gx * gx + gy * gy) * 8 + ax + ay;
}

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
  // stable insertion sort by row_rank
  for (int i = 1; i < t.n; ++i)
    for (int j = i; j > 0 && row_rank(t.o[j][0], t.o[j][1]) < row_rank(t.o[j - 1][0], t.o[j - 1][1]);
         --j)
      for (int k = 0; k < 2; ++k) {
        const signed char v = t.o[j][k];
        t.o[j][k] = t.o[j - 1][k];
        t.o[j - 1][k] = v;
      }
  return t;
}

// Union passes over the half stencil, run in order with a compression between
// them, so that by the later, larger passes most neighbour cells are in A's
// set already and settle from one parent load instead of a root chase and a
// link search.  3D: 0 the face neighbours (one axis off by one), 1 the rest of
// the 3^3 shell, 2 the cells two away along some axis (on C3 the face pass cut
// the union phase from 2.79 to 2.08 ms).  2D: 0 the 3^2 shell, 1 the rest (a
// separate face pass there cost more than it saved).
constexpr int kUnionPasses = 3;

constexpr int union_passes(int D) { return D == 3 ? 3 : 2; }

constexpr int union_pass(int D, int x, int y, int z) {
  const int ax = x < 0 ? -x : x, ay = y < 0 ? -y : y, az = z < 0 ? -z : z;
  if (ax > 1 || ay > 1 || az > 1) return union_passes(D) - 1;
  return D == 3 && ax + ay + az != 1 ? 1 : 0;
}

constexpr bool half_pos(int x, int y, int z) {
  return x > 0 || (x == 0 && (y > 0 || (y == 0 && z > 0)));
}

constexpr OffTab make_half(int D, int pass) {
  OffTab t{};
  const int zr = D == 3 ? 2 : 0;
  for (int x = -2; x <= 2; ++x)
    for (int y = -2; y <= 2; ++y)
      for (int z = -zr; z <= zr; ++z) {
        if (!half_pos(x, y, z) || union_pass(D, x, y, z) != pass) continue;
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
// rows per dimension, and the 3D rows within one cell of the own row (the
// first nine of make_rows(3))
constexpr int kRowsPerDim[2] = {5, 25};
constexpr int kNearRows3 = 9;
static_assert(make_rows(2).n == kRowsPerDim[0] && make_rows(3).n == kRowsPerDim[1], "rows");
static_assert(row_rank(make_rows(3).o[kNearRows3 - 1][0], make_rows(3).o[kNearRows3 - 1][1]) < 8 &&
                  row_rank(make_rows(3).o[kNearRows3][0], make_rows(3).o[kNearRows3][1]) >= 8,
              "the near rows come first");
__constant__ OffTab kHalf[2][kUnionPasses] = {{make_half(2, 0), make_half(2, 1), make_half(2, 2)},
                                              {make_half(3, 0), make_half(3, 1), make_half(3, 2)}};

// Per union pass and stencil row (ox, oy; oy = 0 in 2D, whose rows run along
// the second axis): bit dz + 2 set when the cell at last-axis offset dz is in
// the half stencil and in that pass.
struct PassZ {
  unsigned char m[2][kUnionPasses][5][5];
};

constexpr PassZ make_pass_z() {
  PassZ t{};
  for (int p = 0; p < kUnionPasses; ++p)
    for (int x = -2; x <= 2; ++x)
      for (int y = -2; y <= 2; ++y)
        for (int dz = -2; dz <= 2; ++dz) {
          if (y == 0 && half_pos(x, dz, 0) && union_pass(2, x, dz, 0) == p)
            t.m[0][p][x + 2][2] |= (unsigned char)(1u << (dz + 2));
          if (half_pos(x, y, dz) && union_pass(3, x, y, dz) == p)
            t.m[1][p][x + 2][y + 2] |= (unsigned char)(1u << (dz + 2));
        }
  return t;
}

__constant__ PassZ kPassZ = make_pass_z();
__constant__ OffTab kFullSt[2] = {make_full(2), make_full(3)};

// Per-warp list of candidate rows: row r holds the points lo[r] .. lo[r]+len,
// and pre[r] is the exclusive prefix of the lengths (rows concatenated in
// table order).  Lane r looks its row up, so all lookups are in flight at once.
struct RowList {
  int lo[32];
  int pre[32];
};

template <int D>
__device__ __forceinline__ int build_rows(const gdl::Bufs& B, RowList& RL, const GridView& gv,
                                          const CellXYZ<D>& cc,
                                          const DevParams& P, int lane) {
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
      const int2 rg = gv.span(B, (uint64_t)(rowkey + l0), (uint64_t)(rowkey + l1));
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
  if (P.fast_origin) {
    // o = fl32((lo - centre) + c f) from float pairs: c f_hi by an exact
    // two-product (fma), added to b_hi by an exact two-sum, the small terms
    // (product error, c f_lo, b_lo) summed in float; one final rounding.  The
    // result is within |o| 2^-24 (1 + 2^-20) of the exact value (c < 2^24 is
    // exact in float; the pairs carry 48 bits), which the position error
    // bound (uerr, via ea) covers.
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const float c = (float)(int)cc.c[k];
      const float p = __fmul_rn(c, P.f_hi);
      const float e = __fmaf_rn(c, P.f_hi, -p);
      const float q = __fmul_rn(c, P.f_lo);
      const float a = P.b_hi[k];
      const float s = __fadd_rn(a, p);
      const float v = __fsub_rn(s, a);
      const float t = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(p, v));
      const float low = __fadd_rn(__fadd_rn(t, e), __fadd_rn(q, P.b_lo[k]));
      o[k] = __fadd_rn(s, low);
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < D; ++k)
    o[k] = __double2float_rn(
        __dsub_rn(__dadd_rn(P.lo[k], __dmul_rn((double)cc.c[k], P.f)), P.centre[k]));
}

// A point's position inside its own cell, in cell units (error <= P.uerr).
template <int D, class PP>
__device__ __forceinline__ void frac_pos(const float* xf, const float* o, const PP& P, float* u) {
#pragma unroll
  for (int k = 0; k < D; ++k) u[k] = __fmul_rn(__fsub_rn(xf[k], o[k]), P.inv_f32);
}

// Cell at offset (ox, oy, oz) from the point's cell: 1 every point in it is a
// neighbour (both ways), -1 none is, 0 must be tested.
template <int D, class PP>
__device__ __forceinline__ int classify(const float* u, int ox, int oy, int oz, const PP& P) {
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

// ------------------------------------------------------- thread front ends
// Most work items need little: isolated noise points whose stencil holds fewer
// than minpts points, cells whose neighbour links are found by the first test,
// border points with a handful of candidate cores.  The front-end kernels give
// one thread to each point (k_core_point, k_border_point) or core cell
// (k_union_scan) and finish those cases inline (bounded work per thread); a
// cell that needs more is appended to the heavy list and handled by the
// warp-cooperative *_heavy kernel that follows.  The stencil is walked row by
// row (5 rows in 2D, 25 in 3D, own row first); a row is one contiguous range of
// sorted points, and its non-empty cells are visited through the run structure,
// so empty cells cost nothing.
constexpr int kScanThreadsPerBlock = 256;
// The walk kernels (core count, union scan, border search) take their list
// entries from a global cursor in batches of kWalkBatch, 32 per pass of a
// warp: work is handed out as it is done, so no warp is left with a tail of
// costly entries after the others finish (a static grid-stride split left
// whole SMs idle behind a few slow warps).
constexpr int kWalkBatch = 64;
struct WalkCursor {
  unsigned long long* c;  // kCtrWalkCursor2/3, zero at launch
  int span;               // list entries of this dimension (< 2^31)
  int next, end;          // the warp's batch, relative to its first entry (warp-uniform)
  // the warp's next 32 entries are [next, min(next + 32, end)); false when the
  // list is used up (all lanes call it)
  __device__ __forceinline__ bool advance(int lane) {
    if (next < end) return true;
    unsigned long long got = 0;
    if (lane == 0) got = atomicAdd(c, (unsigned long long)kWalkBatch);
    got = __shfl_sync(kFull, got, 0);
    if (got >= (unsigned long long)span) return false;
    next = (int)got;
    end = span - next > kWalkBatch ? next + kWalkBatch : span;
    return true;
  }
};
template <int D>
__device__ __forceinline__ WalkCursor walk_cursor(const gdl::Bufs& B, int64_t jlo, int64_t jhi) {
  return WalkCursor{B.ctr + (D == 2 ? kCtrWalkCursor2 : kCtrWalkCursor3), (int)(jhi - jlo), 0, 0};
}
// Resident 256-thread blocks per SM the front-end kernels are compiled for
// (register budget 65536 / (256 * blocks) per thread).  These kernels are
// bound by memory latency, so occupancy beats registers; the counts were
// measured on GB300 (a few spilled bytes cost less than a lost block).
#ifndef GD_CORE_MIN_BLOCKS
#define GD_CORE_MIN_BLOCKS 4
#endif
#ifndef GD_UNION_MIN_BLOCKS
#define GD_UNION_MIN_BLOCKS 5
#endif
#ifndef GD_BORDER_MIN_BLOCKS
#define GD_BORDER_MIN_BLOCKS 4
#endif
constexpr int kCoreMinBlocks = GD_CORE_MIN_BLOCKS;
constexpr int kUnionMinBlocks = GD_UNION_MIN_BLOCKS;
constexpr int kBorderMinBlocks = GD_BORDER_MIN_BLOCKS;
// The pair-test budgets of one thread (core count per point, link search per
// cell pair, border search per point) come with the buffers (Bufs::tn_*): the
// context sets them, the autotuner varies them.

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
  // float32-band mode tests from the float32 copy; the float64 coordinates
  // are loaded by the band re-test itself
#pragma unroll
  for (int k = 0; k < D; ++k) {
    if (!F32) x[k] = B.X[k * n + i];
    if (F32 || prune) f[k] = B.Xf[k * n + i];
  }
}

// Stencil rows of a cell: row r of kRows, its first cell's local key, and the
// last-axis cell range [l0, l1] around the cell.
template <int D>
struct RowWalk {
  CellXYZ<D> cc;
  int cl, l0, l1;  // the cell's last-axis index and the stencil's range on that axis
  __device__ __forceinline__ void init(const CellXYZ<D>& c, const DevParams& P) {
    cc = c;
    const int64_t Gl = P.G[D - 1];
    cl = c.c[D - 1];
    l0 = cl - 2 < 0 ? 0 : cl - 2;
    l1 = (int64_t)cl + 2 >= Gl ? (int)(Gl - 1) : cl + 2;
  }
  // local key of row r's first cell, or -1 when the row is outside the grid
  __device__ __forceinline__ int64_t rowkey(const OffTab& T, int r, const DevParams& P) const {
    const int64_t k = offset_key<D>(cc, T.o[r][0], T.o[r][1], 0, P);
    return k < 0 ? k : k - cl;
  }
  // index of row r among the grid's rows (its first cell's key is index * G[D-1]),
  // or -1 when the row is outside the grid
  __device__ __forceinline__ int64_t rowidx(const OffTab& T, int r, const DevParams& P) const {
    const int64_t x = (int64_t)cc.c[0] + T.o[r][0];
    if (x < 0 || x >= P.G[0]) return -1;
    if (D == 2) return x;
    const int64_t y = (int64_t)cc.c[1] + T.o[r][1];
    if (y < 0 || y >= P.G[1]) return -1;
    return x * P.G[1] + y;
  }
};

// next cell of a row walk: [q, end), its last-axis offset from the cell in work
template <bool KEY64>
__device__ __forceinline__ int cell_end(const gdl::Bufs& B, int q) {
  return B.reps[cell_of(B, q) + 1];
}

// Squared largest / smallest distance (plus / minus the position error) along
// one axis from a point at in-cell position a (cell units) to the cell slab at
// offset o.
template <class PP>
__device__ __forceinline__ void axis_terms(float a, int o, const PP& P, float& mx2, float& mn2) {
  const float x = a - (float)o, y = x - 1.0f;
  const float mx = fmaxf(fabsf(x), fabsf(y)) + P.uerr;
  const float mn = fmaxf(fmaxf(-x, y) - P.uerr, 0.0f);
  mx2 = mx * mx;
  mn2 = mn * mn;
}

// undecided cells a point queues before testing them (float64 mode): float64
// tests are costly off the warp-cooperative final flush, and the 3D walks meet
// more undecided cells.  Float32 tests are cheap enough that testing each
// undecided cell at once, with the early exit it allows, wins: that mode keeps
// no queue (lengths measured on GB300).
__host__ __device__ constexpr int core_queue(int d, bool f32) {
  return f32 ? 1 : (d == 2 ? 16 : 24);
}
constexpr int kCoreWarps = kScanThreadsPerBlock / 32;

// Per-warp staging of the final flush (float64 mode): the points whose core
// decision waits on their queued cells, with their instances (lanes of one
// warp may belong to different instances; the predicate constants are read
// from Pv).
template <int D, bool F32>
struct CoreFlushStage {
  double x[32][D];
  float f[32][D];
  int inst[32];
  int cnt[32];    // neighbours counted so far
  int incl[32];   // inclusive prefix of the queued candidate counts
  int nq[32];
};

// Core flags of points in dense cells (at least minpts points: all core, no
// test), with their cells' core counts and smallest core indices.  Every other
// point gets its bit in the walk list's mask (listed in sorted order
// afterwards), so that k_core_point's warps hold only neighbouring points that
// walk.  ONE: a single instance (its parameters are Pv[0]).
template <bool KEY64, bool ONE>
__global__ void k_core_split(const gdl::Bufs B, int64_t n) {
  const int LB = B.Bi->LB;
  const int lane = threadIdx.x & 31;
  unsigned long long dense = 0;
  // two groups of 32 points per warp and pass, their loads issued together
  constexpr int U = 2;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t g0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); g0 < n;
       g0 += U * stride) {
    int m[U], b[U], e[U], mp[U];
    uint32_t id[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = g0 + u * stride + lane;
      const int64_t ic = i < n ? i : n - 1;
      m[u] = cell_of(B, ic);
      id[u] = B.ids[ic];
      mp[u] = B.Pv[ONE ? 0 : (int)(key_at<KEY64>(B, ic) >> LB)].minpts;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      b[u] = B.reps[m[u]];
      e[u] = B.reps[m[u] + 1];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i0 = g0 + u * stride;
      if (i0 >= n) break;  // warp-uniform
      const int64_t i = i0 + lane;
      const bool dn = i < n && e[u] - b[u] >= mp[u];
      if (dn) {
        B.core[i] = 1;
        if (i == b[u]) ++dense;
      }
      // the walk list: every point outside a dense cell
      const unsigned wl = __ballot_sync(kFull, i < n && !dn);
      if (lane == 0) B.lbits[i0 >> 5] = wl;
      const unsigned cm = __ballot_sync(kFull, dn);
      const unsigned grp = run_peers(cm, m[u]);
      if (dn) {
        const unsigned mn = __reduce_min_sync(grp, id[u]);
        if (lane == __ffs(grp) - 1) {
          atomicAdd(B.cellcore + m[u], __popc(grp));
          atomicMin(reinterpret_cast<unsigned*>(B.cellmin) + m[u], mn);
        }
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) dense += __shfl_xor_sync(kFull, dense, o);
  if (lane == 0 && dense) atomicAdd(B.ctr + kCtrDenseCells, dense);
}

// Core flags of the listed points (those outside dense cells, in sorted
// order), one thread per point; warps take the list from the walk cursor.
// Neighbouring lanes hold neighbouring sorted points, mostly of one cell, so
// they walk the same stencil rows in step: their loads coincide and their
// branches agree.  The walk goes row by row, own row first: with cell
// classification, rows and cells wholly inside eps count without tests, those
// wholly outside are skipped.  The classification's per-axis terms are formed
// per row for the fixed axes and per point for the last axis (five pairs in
// per-thread shared memory).  An undecided cell is tested at once in float32
// mode.  In float64 mode undecided cells are queued (shared memory); a full
// queue is tested by its own thread, and what is queued when the walk ends is
// tested by the whole warp together: the lanes whose decision depends on their
// queue pool its candidates and every lane tests one candidate per round (one
// owner's point against one queued point), so the float64 tests run on full
// warps, and owners stop consuming once they reach minpts.  A point whose
// tests pass the budget (or a warp whose pooled candidates pass 32 budgets)
// sends its cell to the warp kernel, which recomputes the whole cell.
// Per-cell core counts and smallest core indices are warp-aggregated atomics
// (cleared before the launch).
//
// Rows [r0, r1) of the stencil.  A walk split in two (3D) first takes the 3x3
// near rows for every listed point (r1 < rows): a point still undecided after
// them keeps its count in lab[] and its bit in fbits, and the second launch
// (r0 > 0) walks the remaining rows for that compacted list only.  Most points
// decide within the near rows, so the second launch's warps hold only the
// points that need the long walk instead of idling beside them (C3: a warp
// ran 13.4 rows where its lanes needed 6.2 on average).
template <int D, bool F32, bool KEY64>
__global__ void __launch_bounds__(kScanThreadsPerBlock, kCoreMinBlocks)
k_core_point(const gdl::Bufs B, int64_t n, int r0, int r1) {
  __shared__ int2 sq[core_queue(D, F32)][kScanThreadsPerBlock];
  // per thread: squared largest / smallest distance terms to the five cell
  // slabs along the last axis (offsets -2..2), kept out of registers
  __shared__ float2 slt[5][kScanThreadsPerBlock];
  __shared__ CoreFlushStage<D, F32> stage[F32 ? 1 : kCoreWarps];
  const OffTab& T = kRows[D - 2];
  const int lane = threadIdx.x & 31;
  const int wbase = threadIdx.x & ~31;
  CoreFlushStage<D, F32>& S = stage[F32 ? 0 : threadIdx.x >> 5];
  const int LB = B.Bi->LB;
  const bool second = r0 > 0;    // the list and counts of a first launch
  const bool split = r1 < T.n;   // a second launch follows
  // this dimension's part of the walk list: 2D instances' points come first
  const int64_t p3 = B.reps[(int64_t)B.ctr[kCtrCells2D]];
  const int64_t L = (int64_t)*B.lcount;
  const int64_t L2 =
      p3 < n ? (int64_t)(second ? bit_rank(B.fbits, B.fpre, p3) : bit_rank(B.lbits, B.lpre, p3))
             : L;
  const int64_t jlo = D == 2 ? 0 : L2, jhi = D == 2 ? L2 : L;
  WalkCursor wc = walk_cursor<D>(B, jlo, jhi);
  Tally t;
  while (wc.advance(lane)) {
    const int64_t j = jlo + wc.next + lane;
    const bool valid = wc.next + lane < wc.end;
    wc.next += 32;
    const int64_t i = valid ? (int64_t)B.blist[j] : 0;
    int m = -1, b = 0;
    bool isc = false, over = false, pend = false;
    int cnt = 0, nq = 0, minpts = 0;
    if (valid && second) cnt = B.lab[i];
    if (valid) {
      m = cell_of(B, i);
      b = B.reps[m];
      const CellCtx cx = cell_ctx<KEY64>(B, b, LB);
      const DevParams& P = *cx.P;
      const PredParams Q = pred_params(P);
      minpts = Q.minpts;
      {
        const GridView gv = view_of(B, P);
        const bool prune = Q.prune != 0;
        RowWalk<D> rw;
        rw.init(decompose<D>(cx.local, P), P);
        double px[D];
        float pf[D];
        load_point<D, F32>(px, pf, B, n, i, prune);
        float u[D];
        if (prune) {
          float o[D];
          cell_origin32<D>(rw.cc, P, o);
          frac_pos<D>(pf, o, Q, u);
#pragma unroll
          for (int j = 0; j < 5; ++j) {
            float a2, b2;
            axis_terms(u[D - 1], j - 2, Q, a2, b2);
            slt[j][threadIdx.x] = make_float2(a2, b2);
          }
        }
        int ptot = 0, budget = B.tn_core;
        // test the points [q, qe) of one cell until the count reaches minpts
        auto test_cell = [&](int q, int qe) {
          for (int qq = q; qq < qe && cnt < Q.minpts; ++qq) {
            if (budget-- == 0) {
              over = true;
              break;
            }
            Cand<D, F32> cd;
            load_cand<D, F32>(cd, B.X, B.Xf, n, qq);
            cnt += pair_test<D, F32>(px, pf, cd, B.X, n, qq, i, true, Q, t) ? 1 : 0;
          }
        };
        auto flush = [&](void) {
          for (int j = 0; j < nq && cnt < Q.minpts && !over; ++j) {
            const int2 c = sq[j][threadIdx.x];
            test_cell(c.x, c.y);
          }
          nq = 0;
          ptot = 0;
        };
        for (int r = r0; r < r1 && cnt < Q.minpts && !over; ++r) {
          float rmx = 0.0f, rmn = 0.0f;
          if (prune) {
#pragma unroll
            for (int k = 0; k < D - 1; ++k) {
              float a2, b2;
              axis_terms(u[k], (int)T.o[r][k], Q, a2, b2);
              rmx += a2;
              rmn += b2;
            }
            if (rmn >= Q.thr_out) continue;  // the whole row is beyond eps
          }
          const int64_t ri = rw.rowidx(T, r, P);
          if (ri < 0) continue;
          const int64_t rk = ri * P.G[D - 1];  // key of the row's first cell
          // one non-empty cell [q, qe) at last-axis offset d from the point's cell
          auto visit = [&](int q, int qe, int d) {
            int cls = 0;
            if (prune) {
              const float2 lt = slt[d + 2][threadIdx.x];
              const float smax = rmx + lt.x, smin = rmn + lt.y;
              cls = smax <= Q.thr_in ? 1 : (smin >= Q.thr_out ? -1 : 0);
            }
            if (cls > 0) {
              cnt += qe - q;
            } else if (cls == 0) {
              if constexpr (F32) {
                test_cell(q, qe);
              } else {
                if (nq == core_queue(D, F32)) flush();
                sq[nq][threadIdx.x] = make_int2(q, qe);
                ++nq;
                ptot += qe - q;
              }
            }
          };
          if (gv.sparse == 0) {
            // cell table: the row's occupied cells from its occupancy bits
            int64_t rr = 0;
            uint32_t mask = gv.occ_cells(B, (uint64_t)rk, rw.l0, rw.l1, rr);
            while (mask && cnt < Q.minpts && !over) {
              const int z = __ffs(mask) - 1;
              mask &= mask - 1;
              visit(B.reps[rr], B.reps[rr + 1], (int)(rw.l0 + z - rw.cl));
              ++rr;
            }
            continue;
          }
          if (gv.sparse == 2) {
            // row table: the row's cells from the first at or after l0 to l1
            const int2 rc = gv.row_cells(B, (uint64_t)ri);
            for (int mq = gv.zlower(B, rc.x, rc.y, rw.l0); mq < rc.y && cnt < Q.minpts && !over;
                 ++mq) {
              const int64_t z = B.cellz[mq];
              if (z > rw.l1) break;
              visit(B.reps[mq], B.reps[mq + 1], (int)(z - rw.cl));
            }
            continue;
          }
          // hash: the row's points, from the first cell at or after l0 to the
          // first beyond l1
          const int2 rp = gv.row(B, (uint64_t)rk);
          if (rp.x == rp.y) continue;
          const int dmax = (int)(rw.l1 - rw.cl);
          for (int q = gv.lower(B, rp.x, rp.y, gv.hi | ((uint64_t)rk + (uint64_t)rw.l0));
               q < rp.y && cnt < Q.minpts && !over;) {
            const int d = (int)((int64_t)((key_at<KEY64>(B, q) & P.kmask) - (uint64_t)rk) - rw.cl);
            if (d > dmax) break;
            const int qe = cell_end<KEY64>(B, q);
            visit(q, qe, d);
            q = qe;
          }
        }
        // what is still queued decides only if it can lift the count to minpts;
        // before a second launch it is always counted (that launch walks the
        // other rows only)
        pend = !over && cnt < Q.minpts && nq > 0 && (split || cnt + ptot >= Q.minpts);
        if (pend) {
#pragma unroll
          for (int k = 0; k < D; ++k) {
            S.x[lane][k] = px[k];
            S.f[lane][k] = pf[k];
          }
          S.inst[lane] = P.inst;
        }
        isc = !over && cnt >= Q.minpts;
      }
    }
    // ---- warp-cooperative final flush (float64 mode)
    const unsigned pm = F32 ? 0u : __ballot_sync(kFull, pend);
    if (!F32 && pm) {
      int tot = 0;
      if (pend)
        for (int j = 0; j < nq; ++j) tot += sq[j][threadIdx.x].y - sq[j][threadIdx.x].x;
      int incl = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += v;
      }
      const int total = __shfl_sync(kFull, incl, 31);
      S.incl[lane] = incl;
      S.nq[lane] = pend ? nq : 0;
      S.cnt[lane] = cnt;
      __syncwarp();
      if (total > 32 * B.tn_core) {
        if (pend) over = true;  // too much for the warp: the warp kernel takes the cell
      } else {
        for (int base = 0; base < total; base += 32) {
          const int c = base + lane;
          if (c < total) {
            // owner: the first lane whose inclusive prefix passes c
            int lo = 0, hi = 31;
            while (lo < hi) {
              const int mid = (lo + hi) >> 1;
              if (S.incl[mid] > c) hi = mid;
              else lo = mid + 1;
            }
            const int ow = lo;
            const PredParams Qo = pred_params(B.Pv[S.inst[ow]]);
            if (S.cnt[ow] < Qo.minpts) {
              int k = c - (ow > 0 ? S.incl[ow - 1] : 0);  // candidate index within the owner's queue
              int qq = -1;
              for (int j = 0; j < S.nq[ow]; ++j) {
                const int2 sg = sq[j][wbase + ow];
                const int len = sg.y - sg.x;
                if (k < len) {
                  qq = sg.x + k;
                  break;
                }
                k -= len;
              }
              if (qq >= 0) {
                Cand<D, F32> cd;
                load_cand<D, F32>(cd, B.X, B.Xf, n, qq);
                // (float64 mode only: the owner's coordinates are staged, no index needed)
                if (pair_test<D, F32>(S.x[ow], S.f[ow], cd, B.X, n, qq, 0, true, Qo, t))
                  atomicAdd(&S.cnt[ow], 1);
              }
            }
          }
          __syncwarp();
          if (__all_sync(kFull, !pend || S.cnt[lane] >= minpts)) break;
        }
        if (pend) {
          cnt = S.cnt[lane];
          isc = cnt >= minpts;
        }
      }
      __syncwarp();
    }
    // undecided after the near rows: on to the second launch
    const bool go_on = split && valid && !over && !isc;
    if (go_on) {
      B.lab[i] = cnt;
      atomicOr(B.fbits + (i >> 5), 1u << (i & 31));
    }
    if (valid && !over && !go_on) B.core[i] = isc ? 1 : 0;
    // per-cell core count and smallest core index, one atomic pair per cell
    // and warp
    const unsigned cm = __ballot_sync(kFull, isc);
    const unsigned grp = run_peers(cm, m);
    if (isc) {
      const unsigned mn = __reduce_min_sync(grp, (unsigned)B.ids[i]);
      if (lane == __ffs(grp) - 1) {
        atomicAdd(B.cellcore + m, __popc(grp));
        atomicMin(reinterpret_cast<unsigned*>(B.cellmin) + m, mn);
      }
    }
    // cells with an undecided point, once per warp
    const unsigned om = __ballot_sync(kFull, over);
    bool lead = false;
    if (over) lead = lane == __ffs(__match_any_sync(om, m)) - 1;
    heavy_push(B, kCtrHeavyCore, lead, m, 0);
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
                                           const PredParams& Q, Tally& t) {
  const bool prune = Q.prune != 0;
  int budget = B.tn_link;
  for (int a = bA; a < eA; ++a) {
    if (!B.core[a]) continue;
    double ax[D];
    float af[D];
    load_point<D, F32>(ax, af, B, n, a, prune);
    if (prune) {
      float u[D];
      frac_pos<D>(af, oA, Q, u);
      const int cls = classify<D>(u, ox, oy, oz, Q);
      if (cls > 0) return 1;
      if (cls < 0) continue;
    }
    for (int q = bB; q < eB; ++q) {
      if (!B.core[q]) continue;
      if (budget-- == 0) return -1;
      Cand<D, F32> cd;
      load_cand<D, F32>(cd, B.X, B.Xf, n, q);
      if (link_test<D, F32>(ax, af, cd, B.X, n, a, q, Q, t, B.asym, B.ctr)) return 1;
    }
  }
  return 0;
}

// bit of offset (ox, oy, oz) in the kHalf[D][pass] table, or -1 if it is not there
struct HalfBits {
  signed char b[2][kUnionPasses][5][5][5];
};

constexpr HalfBits make_half_bits() {
  HalfBits h{};
  for (int d = 0; d < 2; ++d)
    for (int p = 0; p < kUnionPasses; ++p) {
      for (int x = 0; x < 5; ++x)
        for (int y = 0; y < 5; ++y)
          for (int z = 0; z < 5; ++z) h.b[d][p][x][y][z] = -1;
      const OffTab t = make_half(d + 2, p);
      for (int i = 0; i < t.n; ++i)
        h.b[d][p][t.o[i][0] + 2][t.o[i][1] + 2][t.o[i][2] + 2] = (signed char)i;
    }
  return h;
}

__constant__ HalfBits kHalfBits = make_half_bits();

template <int D>
__device__ __forceinline__ int half_bit(int pass, int ox, int oy, int oz) {
  return kHalfBits.b[D - 2][pass][ox + 2][oy + 2][oz + 2];
}

template <int D, bool F32, bool KEY64>
__global__ void __launch_bounds__(kScanThreadsPerBlock, kUnionMinBlocks)
k_union_scan(const gdl::Bufs B, int64_t n, int pass) {
  const OffTab& T = kRows[D - 2];
  const int lane = threadIdx.x & 31;
  const int LB = B.Bi->LB;
  // this dimension's part of the core-cell list: 2D instances' cells come first
  const int64_t M2 = (int64_t)B.ctr[kCtrCells2D];
  const int64_t L = (int64_t)*B.lcount;
  const int64_t L2 = M2 < n ? (int64_t)bit_rank(B.lbits, B.lpre, M2) : L;
  const int64_t jlo = D == 2 ? 0 : L2, jhi = D == 2 ? L2 : L;
  WalkCursor wc = walk_cursor<D>(B, jlo, jhi);
  Tally t;
  while (wc.advance(lane)) {
    const int64_t j = jlo + wc.next + lane;
    const bool valid = wc.next + lane < wc.end;
    wc.next += 32;
    const int64_t m = valid ? (int64_t)B.blist[j] : 0;
    unsigned long long open = 0;
    if (valid) {
      const int b = B.reps[m];
      {
        const int e = B.reps[m + 1];
        const CellCtx cx = cell_ctx<KEY64>(B, b, LB);
        const DevParams& P = *cx.P;
        const PredParams Q = pred_params(P);
        const GridView gv = view_of(B, P);
        RowWalk<D> rw;
        rw.init(decompose<D>(cx.local, P), P);
        float oA[D];
        if (Q.prune) cell_origin32<D>(rw.cc, P, oA);
        // A's parent as the compression before this pass left it: A's root at
        // the start of the pass.  Neighbours' parents were compressed at the
        // same time, so one equal to it puts the cell in A's set however the
        // pass's unions have moved the root since (ra, the current root, is
        // checked too).
        const int ra0 = reinterpret_cast<volatile int*>(B.parent)[m];
        int ra = uf_find(B.parent, (int)m);
        for (int r = 0; r < T.n; ++r) {
          const int ox = T.o[r][0], oy = T.o[r][1];
          // the row's last-axis offsets in this pass (bit dz + 2)
          const uint32_t zm = kPassZ.m[D - 2][pass][ox + 2][oy + 2];
          if (!zm) continue;
          const int64_t rk = rw.rowkey(T, r, P);
          if (rk < 0) continue;
          int64_t z0 = (int64_t)rw.cl - 2 + (__ffs(zm) - 1);
          int64_t z1 = (int64_t)rw.cl - 2 + (31 - __clz(zm));
          z0 = z0 < rw.l0 ? rw.l0 : z0;
          z1 = z1 > rw.l1 ? rw.l1 : z1;
          if (z0 > z1) continue;
          // bit z - z0: cell z of the row is in this pass
          const uint32_t allow = zm >> (int)(z0 - ((int64_t)rw.cl - 2));
          // one cell holding a core point (index c, last-axis offset d).  Its
          // points are looked up only when a link search is needed.
          auto visit_core = [&](int c, int d) {
            // ra: a root of A's set, refreshed only when c's root differs.  A
            // parent equal to ra puts c in A's set from one load (ra stays in
            // A's set whatever is hooked later; the pass before compressed the
            // parents to roots).
            const int pc = reinterpret_cast<volatile int*>(B.parent)[c];
            if (pc == ra || pc == ra0) return;
            const int rc = pc == c ? c : uf_find(B.parent, pc);
            if (rc == ra) return;
            ra = uf_find(B.parent, ra);
            if (rc == ra) return;
            const int q = B.reps[c], qe = B.reps[c + 1];
            const int res = D == 3 ? inline_link<D, F32>(B, n, b, e, q, qe, oA, ox, oy, d, Q, t)
                                   : inline_link<D, F32>(B, n, b, e, q, qe, oA, ox, d, 0, Q, t);
            if (res > 0) {
              uf_union(B.parent, B.cellmin, (int)m, c);
              ra = uf_find(B.parent, ra);
            } else if (res < 0) {
              // the pass masks keep every visited offset in this pass's half
              // stencil
              const int bit = D == 3 ? half_bit<D>(pass, ox, oy, d) : half_bit<D>(pass, ox, d, 0);
              if (bit >= 0) open |= 1ull << bit;
            }
          };
          // a cell of unknown core state
          auto visit = [&](int c, int d) {
            if (B.cellcore[c] > 0) visit_core(c, d);
          };
          if (gv.sparse == 0) {
            // cell table: the cells holding a core point, from the occupancy and
            // core occupancy bits (a cell's index into reps: the rank of the
            // first occupied one plus the occupied cells before it).  Their
            // parents are read together first, through the cache: a parent
            // equal to ra settles the cell even if it is stale, since sets only
            // merge; the others are looked at again from fresh loads.
            int64_t rr = 0;
            const uint32_t mask = gv.occ_cells(B, (uint64_t)rk, z0, z1, rr);
            const uint32_t cm = mask & allow & gv.core_cells(B, (uint64_t)rk, z0, z1);
            uint32_t slow = 0;
#pragma unroll
            for (int z = 0; z < 5; ++z) {
              if ((cm >> z) & 1u) {
                const int64_t r = rr + __popc(mask & ((1u << z) - 1u));
                const int pr = B.parent[r];
                if (pr != ra && pr != ra0) slow |= 1u << z;
              }
            }
            while (slow) {
              const int z = __ffs(slow) - 1;
              slow &= slow - 1;
              const int64_t r = rr + __popc(mask & ((1u << z) - 1u));
              visit_core((int)r, (int)(z0 + z - rw.cl));
            }
            continue;
          }
          if (gv.sparse == 2) {
            // row table: the row's cells with last-axis coordinate in [z0, z1],
            // rows without a core point skipped
            const uint64_t ri = udiv_by((uint64_t)rk, gv.glm, gv.gls);
            if (!gv.core_row_at(B, ri)) continue;
            const int2 rc = gv.row_cells(B, ri);
            for (int mq = gv.zlower(B, rc.x, rc.y, z0); mq < rc.y; ++mq) {
              const int64_t z = B.cellz[mq];
              if (z > z1) break;
              if ((allow >> (int)(z - z0)) & 1u) visit(mq, (int)(z - rw.cl));
            }
            continue;
          }
          const int2 sp = gv.span_row(B, (uint64_t)rk, z0, z1);
          for (int q = sp.x; q < sp.y;) {
            const int c = cell_of(B, q);
            const int qe = B.reps[c + 1];
            const int64_t z = (int64_t)((key_at<KEY64>(B, q) & P.kmask) - (uint64_t)rk);
            if ((allow >> (int)(z - z0)) & 1u) visit(c, (int)(z - rw.cl));
            q = qe;
          }
        }
      }
    }
    heavy_push(B, kCtrHeavyUnion, open != 0, m, open);
  }
  flush_tally(t, B.ctr);
}

// Border labels, one thread per listed non-core point (k_label lists them,
// consecutive lanes holding consecutive sorted points).  Each point walks its
// stencil and takes the smallest cluster id among the cells whose core points
// have it in their neighbourhood (centre = the core point, as the reference's
// expansion queries from the core point).  Cells whose id cannot improve on
// the best so far are skipped; with classification, a cell wholly inside eps
// gives its id without tests and one wholly outside is skipped.  A point whose
// tests pass the budget sends its cell to the warp kernel.
template <int D, bool F32, bool KEY64>
__global__ void __launch_bounds__(kScanThreadsPerBlock, kBorderMinBlocks) k_border_point(const gdl::Bufs B, int64_t n) {
  // per thread: squared largest / smallest distance terms to the five cell
  // slabs along the last axis (offsets -2..2), kept out of registers
  __shared__ float2 slt[5][kScanThreadsPerBlock];
  const OffTab& T = kRows[D - 2];
  const int lane = threadIdx.x & 31;
  const int LB = B.Bi->LB;
  // this dimension's part of the list: 2D instances' points come first
  const int64_t p3 = B.reps[(int64_t)B.ctr[kCtrCells2D]];
  const int64_t L = (int64_t)*B.lcount;
  const int64_t L2 = p3 < n ? (int64_t)bit_rank(B.lbits, B.lpre, p3) : L;
  const int64_t jlo = D == 2 ? 0 : L2, jhi = D == 2 ? L2 : L;
  WalkCursor wc = walk_cursor<D>(B, jlo, jhi);
  Tally t;
  while (wc.advance(lane)) {
    const int64_t j = jlo + wc.next + lane;
    const bool valid = wc.next + lane < wc.end;
    wc.next += 32;
    int m = -1;
    bool over = false;
    if (valid) {
      const int64_t i = (int64_t)B.blist[j];
      m = cell_of(B, i);
      const int b = B.reps[m];
      const CellCtx cx = cell_ctx<KEY64>(B, b, LB);
      const DevParams& P = *cx.P;
      const PredParams Q = pred_params(P);
      const GridView gv = view_of(B, P);
      const bool prune = Q.prune != 0;
      RowWalk<D> rw;
      rw.init(decompose<D>(cx.local, P), P);
      double px[D];
      float pf[D];
      load_point<D, F32>(px, pf, B, n, i, prune);
      float u[D];
      if (prune) {
        float o[D];
        cell_origin32<D>(rw.cc, P, o);
        frac_pos<D>(pf, o, Q, u);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          float a2, b2;
          axis_terms(u[D - 1], k - 2, Q, a2, b2);
          slt[k][threadIdx.x] = make_float2(a2, b2);
        }
      }
      int best = INT_MAX, budget = B.tn_border;
      for (int r = 0; r < T.n && !over; ++r) {
        float rmx = 0.0f, rmn = 0.0f;
        if (prune) {
#pragma unroll
          for (int k = 0; k < D - 1; ++k) {
            float a2, b2;
            axis_terms(u[k], (int)T.o[r][k], Q, a2, b2);
            rmx += a2;
            rmn += b2;
          }
          if (rmn >= Q.thr_out) continue;  // the whole row is beyond eps
        }
        const int64_t ri = rw.rowidx(T, r, P);
        if (ri < 0) continue;
        const int64_t rk = ri * P.G[D - 1];  // key of the row's first cell
        if (gv.sparse == 0) {
          // cell table: visit only the cells holding a core point.  The
          // occupancy, core occupancy and prefix words load together; then the
          // row's cluster ids, together: a row none of whose ids is below best
          // is done without looking at its cells.
          int64_t rr = 0;
          const uint32_t mask = gv.occ_cells(B, (uint64_t)rk, rw.l0, rw.l1, rr);
          uint32_t cm = mask & gv.core_cells(B, (uint64_t)rk, rw.l0, rw.l1);
          int rowmin = INT_MAX;
#pragma unroll
          for (int z = 0; z < 5; ++z)
            if ((cm >> z) & 1u) rowmin = min(rowmin, B.cellcid[rr + __popc(mask & ((1u << z) - 1u))]);
          if (rowmin >= best) continue;
          while (cm && !over) {
            const int z = __ffs(cm) - 1;
            cm &= cm - 1;
            const int64_t rq = rr + __popc(mask & ((1u << z) - 1u));
            const int cB = B.cellcid[rq];
            if (cB >= best) continue;
            int cls = 0;
            if (prune) {
              const int d = (int)(rw.l0 + z - rw.cl);
              const float2 lt = slt[d + 2][threadIdx.x];
              const float smax = rmx + lt.x, smin = rmn + lt.y;
              cls = smax <= Q.thr_in ? 1 : (smin >= Q.thr_out ? -1 : 0);
            }
            if (cls > 0) {
              best = cB;
            } else if (cls == 0) {
              const int q = B.reps[rq], qe = B.reps[rq + 1];
              for (int qq = q; qq < qe; ++qq) {
                if (!B.core[qq]) continue;
                if (budget-- == 0) {
                  over = true;
                  break;
                }
                Cand<D, F32> cd;
                load_cand<D, F32>(cd, B.X, B.Xf, n, qq);
                if (pair_test<D, F32>(px, pf, cd, B.X, n, qq, i, false, Q, t)) {
                  best = cB;
                  break;
                }
              }
            }
          }
          continue;
        }
        if (gv.sparse == 2 && !gv.core_row_at(B, (uint64_t)ri)) continue;
        // one non-empty cell (index c, points [q, qe)) at last-axis offset d;
        // cells without core points have cluster id INT_MAX
        auto visitb = [&](int c, int q, int qe, int d) {
          const int cB = B.cellcid[c];
          if (cB >= best) return;
          int cls = 0;
          if (prune) {
            const float2 lt = slt[d + 2][threadIdx.x];
            const float smax = rmx + lt.x, smin = rmn + lt.y;
            cls = smax <= Q.thr_in ? 1 : (smin >= Q.thr_out ? -1 : 0);
          }
          if (cls > 0) {
            best = cB;  // every point of that cell, a core among them, is in reach
          } else if (cls == 0) {
            for (int qq = q; qq < qe; ++qq) {
              if (!B.core[qq]) continue;
              if (budget-- == 0) {
                over = true;
                break;
              }
              Cand<D, F32> cd;
              load_cand<D, F32>(cd, B.X, B.Xf, n, qq);
              if (pair_test<D, F32>(px, pf, cd, B.X, n, qq, i, false, Q, t)) {
                best = cB;
                break;
              }
            }
          }
        };
        if (gv.sparse == 2) {
          // row table: the row's cells from the first at or after l0 to l1
          const int2 rc = gv.row_cells(B, (uint64_t)ri);
          for (int mq = gv.zlower(B, rc.x, rc.y, rw.l0); mq < rc.y && !over; ++mq) {
            const int64_t z = B.cellz[mq];
            if (z > rw.l1) break;
            visitb(mq, B.reps[mq], B.reps[mq + 1], (int)(z - rw.cl));
          }
          continue;
        }
        // hash: the row's points from the first cell at or after l0
        const int2 rp = gv.row(B, (uint64_t)rk);
        if (rp.x == rp.y) continue;
        const int dmax = (int)(rw.l1 - rw.cl);
        for (int q = gv.lower(B, rp.x, rp.y, gv.hi | ((uint64_t)rk + (uint64_t)rw.l0));
             q < rp.y && !over;) {
          const int d = (int)((int64_t)((key_at<KEY64>(B, q) & P.kmask) - (uint64_t)rk) - rw.cl);
          if (d > dmax) break;
          const int c = cell_of(B, q);
          const int qe = B.reps[c + 1];
          visitb(c, q, qe, d);
          q = qe;
        }
      }
      if (!over) B.lab[i] = best == INT_MAX ? kNoise : best;
    }
    // cells with an undecided point, once per warp
    const unsigned om = __ballot_sync(kFull, over);
    bool lead = false;
    if (over) lead = lane == __ffs(__match_any_sync(om, m)) - 1;
    heavy_push(B, kCtrHeavyBorder, lead, m, 0);
  }
  flush_tally(t, B.ctr);
}

// ------------------------------------------------------------- core flags
// Heavy cells, one warp each: dense cells (>= minpts points) are all core;
// other queued cells stream their candidate rows (5 cells along the last axis
// each, 5 rows in 2D, 25 in 3D, looked up one per lane and concatenated) 32 at
// a time, one candidate per lane, and every staged point of the cell gets
// __ballot_sync + __popc of the lanes holding a neighbour.  The warp stops as
// soon as every staged point has reached minpts (own row first).
template <int D, bool F32, bool KEY64>
__global__ void __launch_bounds__(kCellThreads) k_core_heavy(const gdl::Bufs B, int64_t n) {
  __shared__ WarpStage<D> stage[kWarpsPerBlock];
  __shared__ RowList rows[kWarpsPerBlock];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  WarpStage<D>& S = stage[w];
  RowList& RL = rows[w];
  const int nrows = kRows[D - 2].n;
  const double* __restrict__ X = B.X;
  const float* __restrict__ Xf = B.Xf;
  const int LB = B.Bi->LB;
  int64_t mlo, mhi;
  dim_range<D>(B, mlo, mhi);
  const int64_t W = (int64_t)gridDim.x * kWarpsPerBlock;
  Tally t;
  unsigned long long dense = 0;
  const int64_t H = (int64_t)B.ctr[kCtrHeavyCore];
  for (int64_t h = (int64_t)blockIdx.x * kWarpsPerBlock + w; h < H; h += W) {
    const int64_t m = B.hv_cell[h];
    if (m < mlo || m >= mhi) continue;
    const int b = B.reps[m], e = B.reps[m + 1], sz = e - b;
    const CellCtx cx = cell_ctx<KEY64>(B, b, LB);
    const DevParams& P = *cx.P;
    const PredParams Q = pred_params(P);
    if (sz >= Q.minpts) {
      int mn = INT_MAX;
      for (int i = b + lane; i < e; i += 32) {
        B.core[i] = 1;
        mn = min(mn, (int)B.ids[i]);
      }
      mn = warp_min_i32(mn);
      if (lane == 0) { B.cellcore[m] = sz; B.cellmin[m] = mn; ++dense; }
      continue;
    }
    const GridView gv = view_of(B, P);
    const CellXYZ<D> cc = decompose<D>(cx.local, P);
    const int total = build_rows<D>(B, RL, gv, cc, P, lane);
    int ncore = 0, mn = INT_MAX;
    for (int c0 = 0; c0 < sz; c0 += 32) {
      const int na = min(32, sz - c0);
      if (lane < na) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
          if (!F32) S.x[lane][k] = X[k * n + b + c0 + lane];
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
          bool hit = valid && pair_test<D, F32>(S.x[j], S.f[j], cd, X, n, q, b + c0 + j, true, Q, t);
          unsigned bal = __ballot_sync(kFull, hit);
          if (lane == j) mycnt += __popc(bal);
        }
        done = __all_sync(kFull, lane >= na || mycnt >= Q.minpts);
      }
      const bool isc = lane < na && mycnt >= Q.minpts;
      if (lane < na) B.core[b + c0 + lane] = isc ? 1 : 0;
      if (isc) mn = min(mn, (int)B.ids[b + c0 + lane]);
      ncore += __popc(__ballot_sync(kFull, isc));
      __syncwarp();
    }
    mn = warp_min_i32(mn);
    if (lane == 0) { B.cellcore[m] = ncore; B.cellmin[m] = mn; }
  }
  flush_tally(t, B.ctr);
  if (lane == 0 && dense) atomicAdd(B.ctr + kCtrDenseCells, dense);
}

// ------------------------------------------------------------- union-find
// Union-find roots, the mask of the core-cell list (cells with a core point,
// listed in order for k_union_scan; a word per warp over [0, n)), and the
// core occupancy bit of every core cell's cell-table (row-table) entry, so the
// link and border searches skip cells (rows) without core points without
// looking them up.
template <bool KEY64>
__global__ void k_parent_init(const gdl::Bufs B, int64_t n) {
  const int64_t M = *B.M;
  const int lane = threadIdx.x & 31;
  const int LB = B.Bi->LB;
  // words of the mask beyond the cells are cleared before the launch
  for (int64_t m0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); m0 < M;
       m0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = m0 + lane;
    bool f = false;
    if (m < M) {
      B.parent[m] = (int)m;
      f = B.cellcore[m] > 0;
      if (f && B.occ_words) {
        const uint64_t key = key_at<KEY64>(B, B.reps[m]);
        const DevParams& P = B.Pv[(int)(key >> LB)];
        if (P.sparse != 1) {
          const uint64_t local = key & P.kmask;
          const int a = P.dim - 2;
          const uint64_t idx =
              P.occ_off + (P.sparse == 2 ? udiv_by(local, P.dm[a], P.ds[a]) : local);
          atomicOr(B.cocc + (idx >> 5), 1u << (idx & 31));
        }
      }
    }
    const unsigned bl = __ballot_sync(kFull, f);
    if (lane == 0) B.lbits[m0 >> 5] = bl;
  }
}

// Heavy link searches, one warp per queued cell A: for each still-open
// half-stencil neighbour B (pass 0: offsets within +-1, pass 1: the rest) whose
// core points are in another component, look for one core-core pair that are
// neighbours both ways (lanes over B's points, A's core points broadcast) and
// unite the two cells.
template <int D, bool F32, bool KEY64>
__global__ void __launch_bounds__(kCellThreads) k_union_heavy(const gdl::Bufs B, int64_t n, int pass) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const double* __restrict__ X = B.X;
  const float* __restrict__ Xf = B.Xf;
  const int LB = B.Bi->LB;
  int64_t mlo, mhi;
  dim_range<D>(B, mlo, mhi);
  const int64_t W = (int64_t)gridDim.x * kWarpsPerBlock;
  const OffTab& T = kHalf[D - 2][pass];
  Tally t;
  const int64_t H = (int64_t)B.ctr[kCtrHeavyUnion];
  for (int64_t h = (int64_t)blockIdx.x * kWarpsPerBlock + w; h < H; h += W) {
    const int64_t m = B.hv_cell[h];
    if (m < mlo || m >= mhi) continue;
    const unsigned long long open = B.hv_mask[h];
    const int b = B.reps[m];
    const int e = B.reps[m + 1];
    const CellCtx cx = cell_ctx<KEY64>(B, b, LB);
    const DevParams& P = *cx.P;
    const PredParams Q = pred_params(P);
    const GridView gv = view_of(B, P);
    const CellXYZ<D> cc = decompose<D>(cx.local, P);
    for (int t0 = 0; t0 < T.n; t0 += 32) {
      const int tt = t0 + lane;
      bool cand = false;
      int bB = 0, eB = 0, cB = 0;
      if (tt < T.n && ((open >> tt) & 1ull)) {
        const int64_t kb = offset_key<D>(cc, T.o[tt][0], T.o[tt][1], T.o[tt][2], P);
        if (kb >= 0) {
          const int2 cb = gv.cell(B, (uint64_t)kb);
          bB = cb.x;
          eB = cb.y;
          if (bB < eB) {
            cB = cell_of(B, bB);
            cand = B.cellcore[cB] > 0 && uf_find(B.parent, cB) != uf_find(B.parent, (int)m);
          }
        }
      }
      unsigned mask = __ballot_sync(kFull, cand);
      while (mask) {
        const int src = __ffs(mask) - 1;
        mask &= mask - 1;
        const int cbB = __shfl_sync(kFull, bB, src);
        const int ceB = __shfl_sync(kFull, eB, src);
        const int ccB = __shfl_sync(kFull, cB, src);
        if (uf_find(B.parent, (int)m) == uf_find(B.parent, ccB)) continue;
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
              if (!F32) ax[k] = X[k * n + a];
              if (F32) af[k] = Xf[k * n + a];
            }
            bool hit = valid && link_test<D, F32>(ax, af, c, X, n, a, q, Q, t, B.asym, B.ctr);
            found = __any_sync(kFull, hit);
          }
        }
        if (found && lane == 0) uf_union(B.parent, B.cellmin, (int)m, ccB);
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
    int ra = uf_find(parent, cell_of(B, a));
    int rb = uf_find(parent, cell_of(B, b));
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

// parent[m] <- root (full path compression)
__global__ void k_compress(const gdl::Bufs B) {
  const int64_t M = *B.M;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    if (B.cellcore[m] == 0) continue;
    B.parent[m] = uf_find(B.parent, (int)m);
  }
}

// every root marks its component's smallest core index (a bit over global
// point indices; cluster numbers are the ranks of these bits)
__global__ void k_roots(const gdl::Bufs B) {
  const int64_t M = *B.M;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    if (B.cellcore[m] == 0) continue;
    if (uf_find(B.parent, (int)m) == (int)m) {
      const uint32_t cm = (uint32_t)B.cellmin[m];
      atomicOr(B.fbits + (cm >> 5), 1u << (cm & 31));
    }
  }
}

// Per cell: the cluster id of its core points (the rank of its root's mark,
// less the marks of the instances before it: cluster numbers restart at 0 in
// every instance), INT_MAX without core points.
template <bool KEY64>
__global__ void k_cell_ids(const gdl::Bufs B) {
  const int LB = B.Bi->LB;
  const int64_t M = *B.M;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    int cid = INT_MAX;
    if (B.cellcore[m] > 0) {
      const uint64_t key = key_at<KEY64>(B, B.reps[m]);
      const DevParams& P = B.Pv[(int)(key >> LB)];
      const int64_t root_min = B.cellmin[uf_find(B.parent, (int)m)];
      cid = (int)(bit_rank(B.fbits, B.fpre, root_min) - bit_rank(B.fbits, B.fpre, P.pt_off));
    }
    B.cellcid[m] = cid;
  }
}

// The mask of the border-search list: every non-core point (listed in sorted
// order afterwards, so neighbouring list entries are neighbouring points, 2D
// instances' first), a word per warp.
__global__ void k_label(const gdl::Bufs B, int64_t n) {
  const int lane = threadIdx.x & 31;
  // four groups of 32 points per warp and pass, their loads issued together
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t g0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); g0 < n;
       g0 += U * stride) {
    uint8_t c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = g0 + u * stride + lane;
      c[u] = i < n ? B.core[i] : (uint8_t)1;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i0 = g0 + u * stride;
      if (i0 >= n) break;  // warp-uniform
      const unsigned nc = __ballot_sync(kFull, !c[u]);
      if (lane == 0) B.lbits[i0 >> 5] = nc;
    }
  }
}

// Border points: one warp per cell with non-core points (only non-dense cells
// have any).  Each staged non-core point takes the smallest cluster id among
// the cells whose core points have it in their neighbourhood (centre = the core
// point, as the reference's expansion queries from the core point).  Lanes look
// the stencil cells up in parallel; cells whose cluster id cannot improve any
// staged point are skipped.
template <int D, bool F32, bool KEY64>
__global__ void __launch_bounds__(kCellThreads) k_border_heavy(const gdl::Bufs B, int64_t n) {
  __shared__ WarpStage<D> stage[kWarpsPerBlock];
  __shared__ int sIdx[kWarpsPerBlock][32];
  const int LB = B.Bi->LB;
  int64_t mlo, mhi;
  dim_range<D>(B, mlo, mhi);
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
    if (m < mlo || m >= mhi) continue;
    const int b = B.reps[m], e = B.reps[m + 1];
    const CellCtx cx = cell_ctx<KEY64>(B, b, LB);
    const DevParams& P = *cx.P;
    const PredParams Q = pred_params(P);
    const GridView gv = view_of(B, P);
    const CellXYZ<D> cc = decompose<D>(cx.local, P);
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
          if (!F32) S.x[slot][k] = X[k * n + i];
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
            const int2 cb = gv.cell(B, (uint64_t)kb);
            bB = cb.x;
            eB = cb.y;
            if (bB < eB) {
              cid = B.cellcid[cell_of(B, bB)];  // INT_MAX without core points
              has = cid != INT_MAX;
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
              bool hit = valid && pair_test<D, F32>(S.x[j], S.f[j], c, X, n, q, sIdx[w][j], false, Q, t);
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

// labels back to the caller's point order (core points: their cell's cluster;
// the others: the border search's label or NOISE); counts
__global__ void k_scatter_labels(const gdl::Bufs B, int64_t n, int* __restrict__ out,
                                 uint8_t* __restrict__ core_out) {
  unsigned long long nn = 0, nc = 0;
  // four points per thread and pass, in straight-line phases so that each
  // phase's loads are in flight together: ids, core flags, run words; then
  // both candidate labels (the border search's, and the cell's cluster for a
  // core point); then the stores
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += U * stride) {
    uint32_t j[U], rb[U], rp[U];
    uint8_t c[U];
    int l[U], lc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + u * stride < n ? i0 + u * stride : n - 1;
      j[u] = B.ids[i];
      c[u] = B.core[i];
      rb[u] = B.runbits[i >> 5];
      rp[u] = B.runpre[i >> 5];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + u * stride < n ? i0 + u * stride : n - 1;
      const int m = (int)(rp[u] + (uint32_t)__popc(rb[u] & (0xffffffffu >> (31 - (i & 31))))) - 1;
      l[u] = B.lab[i];
      lc[u] = B.cellcid[m];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i0 + u * stride >= n) continue;
      const int lab = c[u] ? lc[u] : l[u];
      out[j[u]] = lab;
      if (core_out) core_out[j[u]] = c[u];
      nn += lab == kNoise;
      nc += c[u];
    }
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

// clusters of every instance: the root marks in its range of global indices
__global__ void k_cluster_counts(const gdl::Bufs B, int K, int64_t* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
    const InstDesc I = B.inst[i];
    out[i] = (int64_t)bit_rank(B.fbits, B.fpre, I.pt_off + I.n) -
             (int64_t)bit_rank(B.fbits, B.fpre, I.pt_off);
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

int grids(const Bufs& B, int K, int nchunks, double mult2, double mult3, uint64_t dense_floor,
          uint64_t dense_per_point, cudaStream_t s) {
  k_bbox_init<<<(K + 255) / 256, 256, 0, s>>>(B, K);
  if (nchunks > 0) k_bbox_chunk<<<nchunks, kBboxThreads, 0, s>>>(B);
  k_params_inst<<<(K + 127) / 128, 128, 0, s>>>(B, K, mult2, mult3, dense_floor, dense_per_point);
  k_layout<<<1, 1024, 0, s>>>(B, K);
  return 3 + (nchunks > 0 ? 1 : 0);
}

int keys(const Bufs& B, bool key64, int nchunks, void* keys_out, cudaStream_t s) {
  if (nchunks <= 0) return 0;
  if (key64)
    k_keys<unsigned long long><<<nchunks, 256, 0, s>>>(B, static_cast<unsigned long long*>(keys_out));
  else
    k_keys<uint32_t><<<nchunks, 256, 0, s>>>(B, static_cast<uint32_t*>(keys_out));
  return 1;
}

int gather(const Bufs& B, bool key64, int64_t n, bool xf, bool one, int sms, cudaStream_t s) {
  const int g = grid_for(n, 256, sms, 8);
  using U64 = unsigned long long;
#define GD_GATHER(KEY, XF)                                                  \
  do {                                                                      \
    if (one) k_gather<KEY, XF, true><<<g, 256, 0, s>>>(B, n);               \
    else k_gather<KEY, XF, false><<<g, 256, 0, s>>>(B, n);                  \
  } while (0)
  if (key64) {
    if (xf) GD_GATHER(U64, true);
    else GD_GATHER(U64, false);
  } else {
    if (xf) GD_GATHER(uint32_t, true);
    else GD_GATHER(uint32_t, false);
  }
#undef GD_GATHER
  return 1;
}

// kernels of one exclusive scan over nw words
static int scan_launches(int64_t nw) { return gdprim::scan_launches(nw); }

// the set bits of B.lbits over [0, n) listed in order into B.blist, their
// count in *B.lcount
static int list_bits(const Bufs& B, int64_t n, int sms, void* scan_temp, cudaStream_t s) {
  const int64_t nw = (n + 31) / 32;
  gdprim::exclusive_scan_popc(B.lbits, B.lpre, nw, scan_temp, B.lcount, s, B.ctr + kCtrWaitTimeouts);
  gdprim::compact_bits(B.lbits, B.lpre, nw, B.blist, sms, s);
  return scan_launches(nw) + (nw > 0 ? 1 : 0);
}

int runs(const Bufs& B, bool key64, int64_t n, bool mixed, int sms, void* scan_temp,
         cudaStream_t s) {
  const int g = grid_for(n, 256, sms, 8);
  const int64_t nw = (n + 31) / 32;
  if (key64) k_run_bits<unsigned long long><<<g, 256, 0, s>>>(
      static_cast<const unsigned long long*>(B.keys), n, B.runbits);
  else k_run_bits<uint32_t><<<g, 256, 0, s>>>(static_cast<const uint32_t*>(B.keys), n, B.runbits);
  gdprim::exclusive_scan_popc(B.runbits, B.runpre, nw, scan_temp, B.M, s, B.ctr + kCtrWaitTimeouts);
  gdprim::compact_bits(B.runbits, B.runpre, nw, reinterpret_cast<uint32_t*>(B.reps), sms, s);
  if (key64) k_runs_finish<unsigned long long><<<1, 32, 0, s>>>(B, n, mixed ? 1 : 0);
  else k_runs_finish<uint32_t><<<1, 32, 0, s>>>(B, n, mixed ? 1 : 0);
  return 3 + scan_launches(nw);
}

int cell_counts(const Bufs& B, bool key64, int64_t n, int sms, cudaStream_t s) {
  if (key64) k_cell_counts<unsigned long long><<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
  else k_cell_counts<uint32_t><<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
  return 1;
}

int start_fill(const Bufs& B, int K, cudaStream_t s) {
  k_start_fill<<<(K + 127) / 128, 128, 0, s>>>(B, K);
  return 1;
}

int occ_rank(const Bufs& B, int K, void* scan_temp, cudaStream_t s) {
  if (!B.occ_words) return 0;
  gdprim::exclusive_scan_popc(B.occ, B.wpre, (int64_t)B.occ_words, scan_temp, nullptr, s, B.ctr + kCtrWaitTimeouts);
  k_rank_off<<<(K + 127) / 128, 128, 0, s>>>(B, K);
  return scan_launches((int64_t)B.occ_words) + 1;
}

int hash_insert(const Bufs& B, bool key64, int64_t n, int sms, cudaStream_t s) {
  if (key64) k_row_hash<unsigned long long><<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
  else k_row_hash<uint32_t><<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
  return 1;
}

#define GD_L1(D, f32, key64, KERNEL, GRID, THREADS, ...)                          \
  do {                                                                            \
    if (f32) {                                                                    \
      if (key64) KERNEL<D, true, true><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);     \
      else KERNEL<D, true, false><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);          \
    } else {                                                                      \
      if (key64) KERNEL<D, false, true><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);    \
      else KERNEL<D, false, false><<<GRID, THREADS, 0, s>>>(__VA_ARGS__);         \
    }                                                                             \
  } while (0)

// one launch per dimension present (bit 0: 2D instances, bit 1: 3D instances)
#define GD_LAUNCH_DIMS(dims, f32, key64, KERNEL, GRID, THREADS, ...)              \
  do {                                                                            \
    if ((dims) & 1) GD_L1(2, f32, key64, KERNEL, GRID, THREADS, __VA_ARGS__);     \
    if ((dims) & 2) GD_L1(3, f32, key64, KERNEL, GRID, THREADS, __VA_ARGS__);     \
  } while (0)

static int per_dim(int dims) { return ((dims & 1) ? 1 : 0) + ((dims & 2) ? 1 : 0); }

int core(const Bufs& B, int64_t n, int dims, bool f32, bool key64, bool one, int sms,
         void* scan_temp, cudaStream_t s) {
  cudaMemsetAsync(B.ctr + kCtrHeavyCore, 0, 8, s);
  // per-cell core counts (0) and smallest core indices (0xffffffff as unsigned)
  cudaMemsetAsync(B.cellcore, 0, (size_t)n * 4, s);
  cudaMemsetAsync(B.cellmin, 0xff, (size_t)n * 4, s);
  // dense cells at once; the other points listed in sorted order for the walk
  const int g = grid_for(n, 256, sms, 8);
  if (key64) {
    if (one) k_core_split<true, true><<<g, 256, 0, s>>>(B, n);
    else k_core_split<true, false><<<g, 256, 0, s>>>(B, n);
  } else {
    if (one) k_core_split<false, true><<<g, 256, 0, s>>>(B, n);
    else k_core_split<false, false><<<g, 256, 0, s>>>(B, n);
  }
  int L = 1 + list_bits(B, n, sms, scan_temp, s);
  cudaMemsetAsync(B.ctr + kCtrWalkCursor2, 0, 16, s);
  // 3D walks split after the 3x3 near rows (the first nine of kRows)
  const int rows2 = kRowsPerDim[0], rows3 = kRowsPerDim[1], near3 = kNearRows3;
  if (dims & 2) cudaMemsetAsync(B.fbits, 0, (size_t)B.nw * 4, s);
  if (dims & 1) GD_L1(2, f32, key64, k_core_point, sms * 8, kScanThreadsPerBlock, B, n, 0, rows2);
  if (dims & 2) {
    GD_L1(3, f32, key64, k_core_point, sms * 8, kScanThreadsPerBlock, B, n, 0, near3);
    // the undecided 3D points, listed in sorted order
    gdprim::exclusive_scan_popc(B.fbits, B.fpre, B.nw, scan_temp, B.lcount, s,
                                B.ctr + kCtrWaitTimeouts);
    gdprim::compact_bits(B.fbits, B.fpre, B.nw, B.blist, sms, s);
    cudaMemsetAsync(B.ctr + kCtrWalkCursor3, 0, 8, s);
    GD_L1(3, f32, key64, k_core_point, sms * 8, kScanThreadsPerBlock, B, n, near3, rows3);
    L += scan_launches(B.nw) + 2;
  }
  GD_LAUNCH_DIMS(dims, f32, key64, k_core_heavy, sms * 8, kCellThreads, B, n);
  return L + 2 * per_dim(dims);
}

int unite(const Bufs& B, int64_t n, int dims, bool f32, bool key64, int sms, void* scan_temp,
          cudaStream_t s) {
  if (B.occ_words) cudaMemsetAsync(B.cocc, 0, B.occ_words * 4, s);
  cudaMemsetAsync(B.lbits, 0, (size_t)B.nw * 4, s);
  if (key64) k_parent_init<true><<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B, n);
  else k_parent_init<false><<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B, n);
  int L = 1 + list_bits(B, n, sms, scan_temp, s);
  int launched = 0;
  for (int pass = 0; pass < kUnionPasses; ++pass) {
    // the dimensions that have this pass
    const int pd = dims & ((pass < union_passes(2) ? 1 : 0) | (pass < union_passes(3) ? 2 : 0));
    if (!pd) continue;
    cudaMemsetAsync(B.ctr + kCtrHeavyUnion, 0, 8, s);
    cudaMemsetAsync(B.ctr + kCtrWalkCursor2, 0, 16, s);
    GD_LAUNCH_DIMS(pd, f32, key64, k_union_scan, sms * 8, kScanThreadsPerBlock, B, n, pass);
    GD_LAUNCH_DIMS(pd, f32, key64, k_union_heavy, sms * 8, kCellThreads, B, n, pass);
    // every parent to its root: the next pass then finds most neighbours in
    // A's set from one load (parent[q] == A's root).  After the last pass the
    // root marks and cluster ids find their roots themselves.
    const bool last = pass == kUnionPasses - 1 ||
                      !(dims & ((pass + 1 < union_passes(2) ? 1 : 0) |
                                (pass + 1 < union_passes(3) ? 2 : 0)));
    if (!last) k_compress<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
    launched += 2 * per_dim(pd) + (last ? 0 : 1);
  }
  k_asym_resolve<<<1, 32, 0, s>>>(B);
  return L + launched + 1;
}

int roots(const Bufs& B, bool key64, int64_t n, int sms, void* scan_temp, cudaStream_t s) {
  cudaMemsetAsync(B.fbits, 0, (size_t)(B.nwf + 1) * 4, s);
  k_roots<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
  // total clusters into the small block (read with the counters)
  gdprim::exclusive_scan_popc(B.fbits, B.fpre, B.nwf, scan_temp, B.K, s, B.ctr + kCtrWaitTimeouts);
  if (key64) k_cell_ids<true><<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
  else k_cell_ids<false><<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B);
  return 2 + scan_launches(B.nwf);
}

int label(const Bufs& B, int64_t n, int sms, void* scan_temp, cudaStream_t s) {
  k_label<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B, n);
  return 1 + list_bits(B, n, sms, scan_temp, s);
}

int border(const Bufs& B, int64_t n, int dims, bool f32, bool key64, int sms, cudaStream_t s) {
  cudaMemsetAsync(B.ctr + kCtrHeavyBorder, 0, 8, s);
  cudaMemsetAsync(B.ctr + kCtrWalkCursor2, 0, 16, s);
  GD_LAUNCH_DIMS(dims, f32, key64, k_border_point, sms * 8, kScanThreadsPerBlock, B, n);
  GD_LAUNCH_DIMS(dims, f32, key64, k_border_heavy, sms * 8, kCellThreads, B, n);
  return 2 * per_dim(dims);
}

int scatter_labels(const Bufs& B, int64_t n, int* out, uint8_t* core_out, int sms,
                   cudaStream_t s) {
  k_scatter_labels<<<grid_for(n, 256, sms, 8), 256, 0, s>>>(B, n, out, core_out);
  return 1;
}

int cluster_counts(const Bufs& B, int K, int64_t* out, cudaStream_t s) {
  k_cluster_counts<<<(K + 255) / 256, 256, 0, s>>>(B, K, out);
  return 1;
}

}  // namespace gdl
