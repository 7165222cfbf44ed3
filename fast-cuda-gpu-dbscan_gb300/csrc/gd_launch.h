// gd_launch.h -- host launchers for the kernels in gd_pipeline.cu.
//
// One run clusters K >= 1 independent instances together.  Their points are
// concatenated (instance i owns global point indices [pt_off_i, pt_off_i+n_i));
// every cell key carries the instance id in its high bits, so one sort, one
// cell list and one launch per phase serve all instances.  Instances are
// ordered 2D first: cells [0, M2) belong to 2D instances, [M2, M) to 3D ones,
// and each cell phase runs one launch per dimension present.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gd_internal.cuh"

namespace gdl {

// Device buffers of one run (see the layout in gd_internal.cuh).  Passed by
// value to the kernels.
struct Bufs {
  const double* coords = nullptr;       // concatenated input, row-major per instance
  const gd::InstDesc* inst = nullptr;   // K instance descriptions
  const gd::Chunk* chunks = nullptr;    // point runs, one instance each
  gd::DevParams* Pv = nullptr;          // K per-instance grid/predicate parameters
  gd::BatchInfo* Bi = nullptr;          // run layout
  long long* bbox = nullptr;            // K x 6 ordered-int bounds
  const void* keys = nullptr;   // sorted cell keys: u32 or u64 (BatchInfo::key64)
  uint32_t* ids = nullptr;      // global point index per sorted position
  int* reps = nullptr;          // M+1 first positions of the non-empty cells
  uint32_t* M = nullptr;        // number of non-empty cells (device scalar, runpre[nw])
  // Bit masks over sorted positions (or cells), nw = ceil(n / 32) words each,
  // with per-word exclusive prefix counts (nw + 1 entries; the last one is the
  // total): a position's rank among the set bits is pre[i / 32] + the set bits
  // below it in its word (bit_rank).
  uint32_t* runbits = nullptr;  // 1 where a cell starts: cell index of i = rank(i + 1) - 1
  uint32_t* runpre = nullptr;
  uint32_t* lbits = nullptr;    // membership of the current walk list (points or cells)
  uint32_t* lpre = nullptr;
  uint32_t* fbits = nullptr;    // n+1 bits over global point indices: 1 at the smallest
  uint32_t* fpre = nullptr;     // core index of each cluster (cluster number = rank)
  int64_t nw = 0;               // words of runbits / lbits
  int64_t nwf = 0;              // words of fbits
  uint32_t* start = nullptr;    // row tables: first cell (index into reps) per row, after
                                // the scan; other instances: one entry holding their cells
  uint32_t* cellz = nullptr;    // per non-empty cell: its last-axis coordinate
  uint32_t* occ = nullptr;      // occupancy bit per cell (cell tables) or row (row tables)
  uint32_t* cocc = nullptr;     // the same for cells / rows holding a core point (after
                                // the core phase; border search)
  uint32_t* wpre = nullptr;     // per occ word: set bits in the words before it
  uint64_t occ_words = 0;       // words of occ (and of cocc, wpre); 0 without tables
  unsigned long long* hkeys = nullptr;  // sparse grids: row hash slots (key of the row's first cell)
  uint32_t* hvals = nullptr;            // sparse grids: row hash slots (begin, end) pairs
  uint32_t hmask = 0;                   // sparse grids: slots - 1
  double* X = nullptr;          // sorted float64 coordinates, max_dim x n
  float* Xf = nullptr;          // sorted centred float32 coordinates, max_dim x n
  uint8_t* core = nullptr;      // core flag per sorted position
  int* cellcore = nullptr;      // per cell m: number of core points
  int* cellmin = nullptr;       // per cell m: smallest global index of a core point
  int* parent = nullptr;        // per cell m: union-find parent (a cell index)
  int* cellcid = nullptr;       // per cell m: cluster id of its core points (INT_MAX: none)
  int* lab = nullptr;           // label per sorted position
  int* asym = nullptr;          // kAsymCap (from, to) sorted-position pairs
  uint32_t* blist = nullptr;    // the current walk list (set bits of lbits in order: sorted
                                // positions or cells, 2D instances' first), capacity n
  uint32_t* lcount = nullptr;   // device scalar: list length (lpre[nw])
  uint32_t* K = nullptr;        // device scalar: clusters of the run
  int* hv_cell = nullptr;       // heavy-work list: cell index m (capacity n)
  unsigned long long* hv_mask = nullptr;  // heavy-work list: stencil offsets still open
  unsigned long long* ctr = nullptr;      // gd::Counter
  // pair-test budgets of one thread before its work goes to a warp kernel
  // (core count per point, link search per cell pair, border search per point)
  int tn_core = 256, tn_link = 48, tn_border = 160;
};

// Words of the occupancy buffer (occ | cocc | wpre) for W occupancy words, and
// the offset of wpre: 256-byte aligned, as the scan reads it in 16-byte vectors.
inline uint64_t occ_wpre_offset(uint64_t W) { return (2 * W + 63) & ~uint64_t(63); }
inline uint64_t occ_buffer_words(uint64_t W) { return occ_wpre_offset(W) + W; }

// The bit masks of a run of n points (runbits, runpre, lbits, lpre, fbits,
// fpre) in one buffer: each array nw + 1 (fbits, fpre: nwf + 1) words, at
// 256-byte aligned offsets.
struct BitLayout {
  int64_t nw = 0, nwf = 0;
  uint64_t off[6] = {};
  uint64_t words = 0;
};
constexpr BitLayout bit_layout(int64_t n) {
  BitLayout L;
  L.nw = (n + 31) / 32;
  L.nwf = (n + 1 + 31) / 32;
  uint64_t at = 0;
  for (int a = 0; a < 6; ++a) {
    L.off[a] = at;
    at += ((uint64_t)(a < 4 ? L.nw : L.nwf) + 1 + 63) & ~uint64_t(63);
  }
  L.words = at;
  return L;
}
// points the Bufs at the bit masks in `words` (bit_layout(n).words words)
inline void set_bits(Bufs& B, uint32_t* words, int64_t n) {
  const BitLayout L = bit_layout(n);
  B.nw = L.nw;
  B.nwf = L.nwf;
  B.runbits = words + L.off[0];
  B.runpre = words + L.off[1];
  B.lbits = words + L.off[2];
  B.lpre = words + L.off[3];
  B.fbits = words + L.off[4];
  B.fpre = words + L.off[5];
  B.M = B.runpre + L.nw;
  B.lcount = B.lpre + L.nw;
}

// Host launchers.  Each returns the number of kernels it launched.
// per-instance bounding boxes, grids and the run layout
int grids(const Bufs& B, int K, int nchunks, double mult2, double mult3, uint64_t dense_floor,
          uint64_t dense_per_point, cudaStream_t s);
// cell keys in global point order (width from the run layout)
int keys(const Bufs& B, bool key64, int nchunks, void* keys_out, cudaStream_t s);
// sorted float64 (and centred float32) coordinates; one: a single instance
int gather(const Bufs& B, bool key64, int64_t n, bool xf, bool one, int sms, cudaStream_t s);
// cell starts: run bits and their ranks, reps, the cell count M, and the split
// between 2D and 3D cells (mixed: a run holding both)
int runs(const Bufs& B, bool key64, int64_t n, bool mixed, int sms, void* scan_temp,
         cudaStream_t s);
// occupancy bits, row-table cell counts, cellz, each instance's first and last cells
int cell_counts(const Bufs& B, bool key64, int64_t n, int sms, cudaStream_t s);
// one-entry start slices (cell counts of instances without a row table); then scan
int start_fill(const Bufs& B, int K, cudaStream_t s);
// occupancy ranks: word prefix counts (scan temp: scan_temp_bytes(occ_words)) and each
// cell table's rank offset
int occ_rank(const Bufs& B, int K, void* scan_temp, cudaStream_t s);
// sparse instances: hash of occupied rows (clear the slots first)
int hash_insert(const Bufs& B, bool key64, int64_t n, int sms, cudaStream_t s);
// cell phases; dims: bit 0 = 2D instances present, bit 1 = 3D; one: a single instance
int core(const Bufs& B, int64_t n, int dims, bool f32, bool key64, bool one, int sms,
         void* scan_temp, cudaStream_t s);
int unite(const Bufs& B, int64_t n, int dims, bool f32, bool key64, int sms, void* scan_temp,
          cudaStream_t s);
// root marks, cluster numbers (total into *B.K), per-cell cluster ids and core
// occupancy bits
int roots(const Bufs& B, bool key64, int64_t n, int sms, void* scan_temp, cudaStream_t s);
// the border-search list (non-core points)
int label(const Bufs& B, int64_t n, int sms, void* scan_temp, cudaStream_t s);
int border(const Bufs& B, int64_t n, int dims, bool f32, bool key64, int sms, cudaStream_t s);
int scatter_labels(const Bufs& B, int64_t n, int* out, uint8_t* core_out, int sms,
                   cudaStream_t s);
// per-instance cluster counts (K entries) from the cluster marks
int cluster_counts(const Bufs& B, int K, int64_t* out, cudaStream_t s);

}  // namespace gdl
