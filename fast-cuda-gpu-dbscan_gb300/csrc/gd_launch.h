// gd_launch.h -- host launchers for the kernels in gd_pipeline.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gd_internal.cuh"

namespace gdl {

// Device buffers of one instance (see the layout in gd_internal.cuh).
struct Bufs {
  gd::DevParams* P = nullptr;
  uint32_t* keys = nullptr;     // sorted cell keys
  uint32_t* ids = nullptr;      // original index per sorted position
  int* reps = nullptr;          // M+1 first positions of the non-empty cells
  uint32_t* M = nullptr;        // number of non-empty cells (device scalar)
  uint32_t* start = nullptr;    // dense cell table, C+1 entries
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
  unsigned long long* ctr = nullptr;  // gd::Counter
};

void bbox(const double* pts, int64_t n, int dim, double* partial, int nblocks, int* flags,
          cudaStream_t s);
void params(const double* partial, int nblocks, int dim, gd::DevParams* P, double eps,
            int minpts, double cell_mult, uint64_t max_cells, const int* flags, cudaStream_t s);
void keys(const double* pts, int64_t n, int dim, const gd::DevParams* P, uint32_t* keys,
          int sms, cudaStream_t s);
void gather(const double* pts, const uint32_t* ids, int64_t n, int dim, bool f32,
            const gd::DevParams* P, double* X, float* Xf, int sms, cudaStream_t s);
void run_flags(const uint32_t* keys, int64_t n, uint32_t* fl, int sms, cudaStream_t s);
void run_scatter(const uint32_t* fl, const uint32_t* pos, int64_t n, int* reps,
                 const uint32_t* Mdev, unsigned long long* ctr, int sms, cudaStream_t s);
void cell_counts(const uint32_t* keys, const int* reps, const uint32_t* Mdev, int64_t n,
                 uint32_t* table, int sms, cudaStream_t s);
void core(const Bufs& B, int64_t n, int dim, bool f32, int sms, cudaStream_t s);
void unite(const Bufs& B, int64_t n, int dim, bool f32, int sms, cudaStream_t s);
void roots(const Bufs& B, int64_t n, int sms, cudaStream_t s);
void label(const Bufs& B, int64_t n, int sms, cudaStream_t s);
void border(const Bufs& B, int64_t n, int dim, bool f32, int sms, cudaStream_t s);
void scatter_labels(const Bufs& B, int64_t n, int* out, uint8_t* core_out, int sms,
                    cudaStream_t s);

}  // namespace gdl
