// gd_launch.h -- host launchers for the kernels in gd_pipeline.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gd_internal.cuh"

namespace gdl {

// Device buffers of one instance (see the layout in gd_internal.cuh).  Passed
// by value to the cell kernels.
struct Bufs {
  gd::DevParams* P = nullptr;
  const void* keys = nullptr;   // sorted cell keys: u32 (dense grid) or u64 (sparse)
  uint32_t* ids = nullptr;      // original index per sorted position
  int* reps = nullptr;          // M+1 first positions of the non-empty cells
  uint32_t* M = nullptr;        // number of non-empty cells (device scalar)
  uint32_t* runfl = nullptr;    // 1 where a cell starts (per sorted position)
  uint32_t* runpos = nullptr;   // exclusive scan of runfl: cell index = runpos+runfl-1
  uint32_t* start = nullptr;    // dense grids: cell table, C+1 entries
  unsigned long long* hkeys = nullptr;  // sparse grids: hash slots (key)
  uint32_t* hvals = nullptr;            // sparse grids: hash slots (cell index m)
  uint32_t hmask = 0;                   // sparse grids: slots - 1
  double* X = nullptr;          // sorted float64 coordinates, D x n
  float* Xf = nullptr;          // sorted centred float32 coordinates, D x n
  uint8_t* core = nullptr;      // core flag per sorted position
  int* cellcore = nullptr;      // per rep: number of core points
  int* cellmin = nullptr;       // per rep: smallest original index of a core point
  int* parent = nullptr;        // per rep: union-find parent
  uint32_t* Fmark = nullptr;    // n: 1 at the smallest core index of each cluster,
                                // then its exclusive scan (cluster ids)
  int* cellcid = nullptr;       // per rep: cluster id of the cell's core points
  int* lab = nullptr;           // label per sorted position
  int* asym = nullptr;          // kAsymCap (from, to) sorted-position pairs
  int* hv_cell = nullptr;       // heavy-work list: cell index m (capacity n)
  unsigned long long* hv_mask = nullptr;  // heavy-work list: stencil offsets still open
  unsigned long long* ctr = nullptr;  // gd::Counter
};

void bbox(const double* pts, int64_t n, int dim, double* partial, int nblocks, int* flags,
          cudaStream_t s);
void params(const double* partial, int nblocks, int dim, gd::DevParams* P, double eps,
            int minpts, double cell_mult, uint64_t max_cells, const int* flags, cudaStream_t s);
// keys: u32 for dense grids, u64 for sparse grids
void keys(const double* pts, int64_t n, int dim, bool sparse, const gd::DevParams* P, void* keys,
          int sms, cudaStream_t s);
void gather(const double* pts, const uint32_t* ids, int64_t n, int dim, bool f32,
            const gd::DevParams* P, double* X, float* Xf, int sms, cudaStream_t s);
void run_flags(const void* keys, bool sparse, int64_t n, uint32_t* fl, int sms, cudaStream_t s);
void run_scatter(const uint32_t* fl, const uint32_t* pos, int64_t n, int* reps,
                 const uint32_t* Mdev, unsigned long long* ctr, int sms, cudaStream_t s);
void cell_counts(const uint32_t* keys, const int* reps, const uint32_t* Mdev, int64_t n,
                 uint32_t* table, int sms, cudaStream_t s);
void hash_insert(const unsigned long long* keys, const int* reps, const uint32_t* Mdev, int64_t n,
                 unsigned long long* hkeys, uint32_t* hvals, uint32_t mask, int sms,
                 cudaStream_t s);
void core(const Bufs& B, int64_t n, int dim, bool f32, bool sparse, int sms, cudaStream_t s);
void unite(const Bufs& B, int64_t n, int dim, bool f32, bool sparse, int sms, cudaStream_t s);
void roots(const Bufs& B, int64_t n, int sms, cudaStream_t s);
void label(const Bufs& B, int64_t n, int sms, cudaStream_t s);
void border(const Bufs& B, int64_t n, int dim, bool f32, bool sparse, int sms, cudaStream_t s);
void scatter_labels(const Bufs& B, int64_t n, int* out, uint8_t* core_out, int sms,
                    cudaStream_t s);

}  // namespace gdl
