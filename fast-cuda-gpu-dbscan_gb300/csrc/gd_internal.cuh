// gd_internal.cuh -- device-side declarations shared by the gbdbscan kernels.
//
// Data layout in HBM for one clustering instance of n points in d dimensions
// (d = 2 or 3), after the index build:
//   keys[n]   u32   fine-cell key of each point, sorted ascending (u64 for
//                   sparse grids)
//   ids[n]    u32   original point index of each sorted position
//   X[k][n]   f64   coordinate k of each sorted position (structure of arrays)
//   start[C+1] i32  dense cell table: points of cell c are start[c]..start[c+1]
//                   (grids up to max(2^26, 8n) cells), or, for larger (sparse)
//                   grids, a hash of the occupied cells' 64-bit keys -> m
//   reps[M+1] i32   sorted position of the first point of every non-empty cell
// Per non-empty cell, indexed by its cell index m (0..M-1, key order; the
// walks reach it from occupancy ranks without loading reps):
//   cellcore[m]  number of core points in the cell
//   cellmin[m]   smallest original index among the cell's core points
//   parent[m]    union-find parent (a cell index)
//   cellcid[m]   cluster id of the cell's core points (INT_MAX: none)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gd {

constexpr int kNoise = -2;            // common.h:8 NOISE
constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// One clustering instance as the caller describes it (uploaded per run).
struct InstDesc {
  int64_t pt_off;      // first point of the instance in the concatenated point list
  int64_t n;           // its points
  int64_t co_off;      // its first coordinate (in doubles) in the concatenated buffer
  double eps;
  int32_t dim;         // 2 or 3
  int32_t minpts;
};

// A run of points of one instance (bbox and key kernels take one block each).
struct Chunk {
  int32_t inst;
  int32_t pad;
  int64_t begin;       // global point indices [begin, end)
  int64_t end;
};
constexpr int64_t kChunkPoints = 8192;

// Whole-run layout, computed on the device after the per-instance grids.
struct BatchInfo {
  int32_t K;           // instances
  int32_t LB;          // local key bits (widest instance grid)
  int32_t IB;          // instance-id bits
  int32_t key64;       // 1: keys are 64-bit
  uint64_t occ_total;  // occupancy bits of all instances (cells of cell tables,
                       // rows of row tables)
  uint64_t start_total;// entries of all start tables (rows+1 per row table, 1 otherwise)
  int32_t any_sparse;  // some instance uses the hash of occupied cells
  int32_t flags;       // OR of the instances' kFlag* bits
  int32_t any_xf;      // some instance wants the centred float32 copy
  int32_t max_dim;
  int32_t K2;          // instances [0, K2) are 2D, [K2, K) 3D
  int32_t band_off;    // some instance has no valid float32 band (all its pairs
                       // take the float64 predicate)
};

// Grid and predicate parameters of one instance, computed on the device from
// its bounding box.
struct DevParams {
  double lo[3];        // per-dimension minimum (grid origin)
  double hi[3];        // per-dimension maximum
  double centre[3];    // bounding-box centre (origin of the float32 copy)
  double f;            // fine cell side
  double inv_f;        // 1 / f
  double eps;          // epsilon
  double eps2;         // fl(eps * eps), the reference's threshold
  double eps2_in;      // float64 d2 <= eps2_in implies the box test passes
  float eps2_lo32;     // float32 d2 below this: certainly a neighbour
  float eps2_hi32;     // float32 d2 above this: certainly not a neighbour
  int64_t G[3];        // cells per dimension
  uint64_t C;          // total cells (G0*G1[*G2])
  uint64_t rows;       // rows: C / G[dim-1]
  int32_t dim;
  int32_t minpts;
  int32_t key_bits;
  int32_t flags;       // kFlag*
  int32_t sparse;      // grid lookup: 0 dense cell table; 2 dense row table (cells
                       // inside a row by binary search); 1 hash of occupied rows
  int32_t prune;       // 1: cell-level inside/outside classification enabled
  float inv_f32;       // fl32(1 / f)
  float uerr;          // bound on the error of a point's in-cell position (cell units)
  float thr_in;        // sum of squared max distances (cell units) below: all neighbours
  float thr_out;       // sum of squared min distances (cell units) above: none
  int64_t pt_off;      // first point (global index)
  int64_t n;           // points
  int64_t co_off;      // first coordinate in the concatenated buffer
  uint64_t occ_off;    // first occupancy bit of this instance (cell table: C+1 bits,
                       // row table: rows+1)
  uint64_t start_off;  // first start-table entry (row table: rows+1 entries, else 1)
  int64_t m0;          // first non-empty cell of the instance (index into reps)
  int64_t m1;          // last non-empty cell of the instance
  int64_t rank_off;    // cell table: a cell's index into reps = occupancy rank + rank_off
  uint64_t kmask;      // mask of the local key bits
  int32_t LB;          // local key bits of the run (copied from BatchInfo)
  int32_t inst;        // instance index
  // exact division of local keys by G[1] and G[2] (multiply-high method, see
  // udiv_magic): multiplier and shift per divisor
  uint64_t dm[2];
  int32_t ds[2];
  // float32 cell origins without float64 arithmetic (cell_origin32): the cell
  // side and lo - centre per axis as float pairs (hi + lo), valid when fast_origin
  float f_hi, f_lo;
  float b_hi[3], b_lo[3];
  int32_t fast_origin;
  // float32 cell keys (k_keys): lo and 1/f in float, and the bound on
  // |t32 - t64| in cell units; a coordinate whose float32 cell position is
  // farther than key_band from a cell boundary takes its cell from it, the
  // others from the float64 formula.  Valid when key_fast.
  float key_lo32[3], key_inv32, key_band;
  int32_t key_fast;
};

// Division by an invariant integer d >= 1 through a multiply-high (Granlund &
// Montgomery, "Division by invariant integers using multiplication", 1994,
// Fig. 4.1, N = 64): with l = ceil(log2 d) and m = floor(2^64 (2^l - d) / d) + 1,
// q = (t + ((k - t) >> 1)) >> (l - 1), t = mulhi(m, k), for every 64-bit k
// (l = 0, i.e. d = 1: q = k).  The multiplier is found by long division.
__host__ __device__ inline void udiv_magic(uint64_t d, uint64_t& m, int32_t& l) {
  l = 0;
  while (l < 64 && (1ull << l) < d) ++l;
  if (l == 0) { m = 0; return; }
  // floor((2^l - d) * 2^64 / d); exact for d < 2^63 (the remainder never overflows)
  uint64_t r = (l == 64 ? 0ull : (1ull << l)) - d, q = 0;
  for (int i = 0; i < 64; ++i) {
    r <<= 1;
    q <<= 1;
    if (r >= d) { r -= d; q |= 1; }
  }
  m = q + 1;
}

__device__ __forceinline__ uint64_t udiv_by(uint64_t k, uint64_t m, int32_t l) {
  if (l == 0) return k;
  const uint64_t t = __umul64hi(m, k);
  return (t + ((k - t) >> 1)) >> (l - 1);
}

// The predicate constants a cell kernel keeps in registers.
struct PredParams {
  double eps, eps2, eps2_in;
  float eps2_lo32, eps2_hi32, uerr, thr_in, thr_out, inv_f32;
  int32_t minpts, prune;
};

__device__ __forceinline__ PredParams pred_params(const DevParams& P) {
  PredParams q;
  q.eps = P.eps;
  q.eps2 = P.eps2;
  q.eps2_in = P.eps2_in;
  q.eps2_lo32 = P.eps2_lo32;
  q.eps2_hi32 = P.eps2_hi32;
  q.uerr = P.uerr;
  q.thr_in = P.thr_in;
  q.thr_out = P.thr_out;
  q.inv_f32 = P.inv_f32;
  q.minpts = P.minpts;
  q.prune = P.prune;
  return q;
}

// A grid too large for a cell table takes a table of its rows when it has at
// most this many rows per point (or the table floor).
constexpr uint64_t kRowsPerPoint = 64;

constexpr int kFlagNonFinite = 1;     // NaN or Inf coordinate
constexpr int kFlagGridTooLarge = 2;  // keys would not fit 62 bits
constexpr int kFlagNoShortcut = 4;    // |x| too large relative to eps for the
                                      // box-test shortcut / float32 filter

// Device counters (u64), zeroed per run.
enum Counter {
  kCtrCells = 0,        // M, number of non-empty cells
  kCtrTests64,          // float64 distance evaluations
  kCtrTests32,          // float32 distance evaluations
  kCtrBand,             // float32 evaluations that fell in the re-test band
  kCtrAsym,             // core pairs that are neighbours in one direction only
  kCtrClusters,         // K
  kCtrCore,             // core points
  kCtrNoise,            // noise points
  kCtrDenseCells,       // cells with >= minpts points
  kCtrAsymEdges,        // one-directional core pairs recorded for the merge replay
  kCtrHeavyCore,        // cells queued for warp-cooperative core counting
  kCtrHeavyUnion,       // cells queued for warp-cooperative link searches
  kCtrHeavyBorder,      // cells queued for warp-cooperative border search
  kCtrCells2D,          // cells of 2D instances (they sort first)
  kCtrWalkCursor2,      // walk-list entries handed out (2D, 3D); cleared before each walk launch
  kCtrWalkCursor3,
  kCtrWaitTimeouts,     // scan / sort launches whose look-back wait gave up (never expected)
  kCtrCount = 17
};

// Capacity of the list of one-directional core-core pairs (see k_asym_resolve).
constexpr int kAsymCap = 2048;

// Hash of occupied cells (sparse grids): open addressing, linear probing.
constexpr unsigned long long kHashEmpty = ~0ull;
__host__ __device__ __forceinline__ uint32_t hash_key(unsigned long long k) {
  return (uint32_t)((k * 0x9E3779B97F4A7C15ull) >> 32);
}

// ---- float64 predicate, bit-exact with the reference's CPU DBSCAN ----------
// Neighbour test with centre p and candidate q: the query box
// [fl(p-eps), fl(p+eps)] with inclusive bounds (cpu-dbscan/Rtree.h:1573-1588)
// and fl(fl(dx*dx) + fl(dy*dy) [+ fl(dz*dz)]) <= fl(eps*eps), dx = fl(p - q)
// (cpu-dbscan/dbscan_rtree_exp.cpp:351-358, 431-432).  The _rn intrinsics keep
// the compiler from fusing multiply-adds, which would change the bits.
template <int D>
__device__ __forceinline__ double dist2_f64(const double* p, const double* q) {
  double a = __dsub_rn(p[0], q[0]);
  double s = __dmul_rn(a, a);
  double b = __dsub_rn(p[1], q[1]);
  s = __dadd_rn(s, __dmul_rn(b, b));
  if (D == 3) {
    double c = __dsub_rn(p[2], q[2]);
    s = __dadd_rn(s, __dmul_rn(c, c));
  }
  return s;
}

template <int D>
__device__ __forceinline__ bool box_f64(const double* p, const double* q, double eps) {
#pragma unroll
  for (int k = 0; k < D; ++k) {
    double lo = __dsub_rn(p[k], eps);
    double hi = __dadd_rn(p[k], eps);
    if (lo > q[k] || q[k] > hi) return false;
  }
  return true;
}

// d2 <= t for a squared distance d2 (a sum of squares of finite values: +0 or
// positive, never -0 or NaN) and any t other than NaN, from the bit patterns:
// non-negative doubles order as their bits do as signed integers, and a
// negative t has a negative pattern, below every d2.  An integer compare keeps
// the test off this GPU's narrow float64 pipe.
__device__ __forceinline__ bool d2_le(double d2, double t) {
  return __double_as_longlong(d2) <= __double_as_longlong(t);
}

// Full predicate given d2 = dist2_f64(p, q).
template <int D, class PP>
__device__ __forceinline__ bool pred_from_d2(double d2, const double* p, const double* q,
                                             const PP& P) {
  if (d2_le(d2, P.eps2_in)) return true;
  if (!d2_le(d2, P.eps2)) return false;
  return box_f64<D>(p, q, P.eps);
}

// ---- union-find over cell reps (lock-free, hooks by (cellmin, position)) ---
__device__ __forceinline__ int uf_find(int* parent, int x) {
  volatile int* par = parent;
  int p = par[x];
  while (p != x) {
    int gp = par[p];
    if (gp != p) par[x] = gp;
    x = p;
    p = gp;
  }
  return x;
}

__device__ __forceinline__ bool uf_less(const int* cellmin, int a, int b) {
  int wa = cellmin[a], wb = cellmin[b];
  return wa < wb || (wa == wb && a < b);
}

__device__ __forceinline__ void uf_union(int* parent, const int* cellmin, int a, int b) {
  while (true) {
    a = uf_find(parent, a);
    b = uf_find(parent, b);
    if (a == b) return;
    if (uf_less(cellmin, b, a)) { int t = a; a = b; b = t; }
    // hook b (the heavier root) under a
    int old = atomicCAS(parent + b, b, a);
    if (old == b) return;
    b = old;
  }
}

}  // namespace gd

// ---- host-side primitive launchers (gd_prims.cu) ---------------------------
namespace gdprim {
// temp bytes needed by exclusive_scan_u32 / exclusive_scan_popc for n
// elements.  Temp memory must be zero when first used and is then kept
// consistent by the primitives themselves (one stream at a time).
size_t scan_temp_bytes(int64_t n);
// kernels one scan of n elements launches
int scan_launches(int64_t n);
// out[i] = sum_{j<i} in[i]; in == out allowed.  Returns the total in *total_dev
// (device pointer, may be null).  timeouts (may be null): incremented when a
// look-back wait gave up (the result is then wrong but every write in bounds).
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, void* temp,
                        uint32_t* total_dev, cudaStream_t s,
                        unsigned long long* timeouts = nullptr);
// pre[w] = number of set bits in words[0, w) (exclusive scan of popcounts),
// total in *total_dev (may be null); words and pre 16-byte aligned, distinct.
void exclusive_scan_popc(const uint32_t* words, uint32_t* pre, int64_t nw, void* temp,
                         uint32_t* total_dev, cudaStream_t s,
                         unsigned long long* timeouts = nullptr);
// the positions of the set bits of words[0, nw) in ascending order:
// out[pre[w] + r] = 32 w + (position of the r-th set bit of word w)
void compact_bits(const uint32_t* words, const uint32_t* pre, int64_t nw, uint32_t* out, int sms,
                  cudaStream_t s);
// temp bytes needed by radix_sort_pairs for n elements (either key width);
// zero when first used, as for the scan
size_t sort_temp_bytes(int64_t n);
// Stable LSD radix sort of (key, value) pairs on the low `bits` key bits,
// K = uint32_t or unsigned long long.  keys/vals: ping-pong buffers [0] and
// [1]; input in [0].  If vals_in_is_iota, vals[0] is not read and the values
// are taken as 0..n-1.  Returns the index (0 or 1) of the buffer that holds the
// result.  timeouts as for the scan.
template <class K>
int radix_sort_pairs(K* keys[2], uint32_t* vals[2], int64_t n, int bits, bool vals_in_is_iota,
                     void* temp, cudaStream_t s, unsigned long long* timeouts = nullptr);
// kernels one radix_sort_pairs call launches
int sort_launches(int64_t n, int bits);
// digit width radix_sort_pairs uses for a `bits`-bit key (8 or 9)
int sort_digit_bits(int bits);
}  // namespace gdprim
