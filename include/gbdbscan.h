/* gbdbscan.h -- C ABI of the GB300-native exact DBSCAN library (libgbdbscan.so).
 *
 * Drop-in for the DBSCAN pipeline of CUDA-DClust+ (l3lackcurtains/fast-cuda-gpu-dbscan).
 * The reference has no library API: it is one program (main.cu) that imports a
 * CSV, builds a grid-tree index on the GPU, expands clusters block by block and
 * merges them on the host, with its configuration fixed at compile time in
 * common.h.  Each entry point below names the reference code it replaces.
 *
 * Conventions kept from the reference:
 *   - points are float64, row-major [n][dim] (main.cu:48-49, 137-139);
 *   - eps and minpts mean what EPS and MINPTS mean in common.h:21-22: a point q
 *     is a neighbour of p when |p - q|^2 <= eps^2 (p itself included), and p is
 *     a core point when it has at least minpts neighbours;
 *   - NOISE = -2 (common.h:8).
 * Changed on purpose:
 *   - labels are per point (the reference writes a sorted unique label list,
 *     dbscan.cu:233-247) and dense: clusters are 0..K-1, numbered in the order of
 *     their smallest core point index, border points take the smallest adjacent
 *     cluster.  The labels equal those of the reference's exact CPU DBSCAN
 *     (cpu-dbscan/dbscan_rtree_exp.cpp) with -1 -> -2 and k -> k-1;
 *   - errors are returned as gd_status codes; nothing calls exit()
 *     (the reference exits in gpuErrchk, common.h:31-40, and on a bin narrower
 *     than eps, main.cu:204-207 -- that restriction does not exist here).
 *
 * Threading: a context is used by one host thread at a time.  Calls are
 * synchronous with respect to the host (they return when results are ready)
 * and run on the context's CUDA stream.
 */
#ifndef GBDBSCAN_H
#define GBDBSCAN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GD_NOISE (-2)       /* common.h:8 */
#define GD_ABI_VERSION 1

typedef enum gd_status {
  GD_OK = 0,
  GD_EINVAL = 1,    /* bad argument: n < 0, dim not 2/3, eps <= 0 or not finite,
                       minpts < 1, NaN/Inf coordinate, NULL pointer */
  GD_ENOMEM = 2,    /* device or host allocation failed */
  GD_ECUDA = 3,     /* CUDA runtime error (message in gd_last_error) */
  GD_ERANGE = 4,    /* the eps-cell grid of this input exceeds the cell-table limit */
  GD_ETIMEOUT = 5,  /* a bounded wait gave up */
  GD_EIO = 6,       /* file could not be opened / parsed */
  GD_ENODEV = 7,    /* no CUDA device, or the device is not sm_103 */
  GD_ESTATE = 8     /* call out of order (e.g. gd_expand before gd_index_build) */
} gd_status;

typedef enum gd_precision {
  GD_PREC_FP64 = 0,      /* every distance test in float64 */
  GD_PREC_FP32_BAND = 1  /* float32 test, float64 re-test inside the proven rounding
                            band; labels identical to GD_PREC_FP64 */
} gd_precision;

typedef struct gd_ctx gd_ctx;

typedef struct gd_points {
  const double* coords; /* n x dim float64, row-major */
  int64_t n;
  int32_t dim;          /* 2 or 3 (common.h:10 DIMENSION) */
  int32_t on_device;    /* 0: host memory; 1: device memory of the context's GPU */
} gd_points;

typedef struct gd_stats {
  int64_t n_points;
  int64_t n_clusters;
  int64_t n_noise;
  int64_t n_core;
  int64_t n_border;
  int64_t n_cells;          /* non-empty grid cells */
  int64_t n_dense_cells;    /* cells with >= minpts points (all core, no test) */
  int64_t tests_fp64;       /* float64 pair evaluations */
  int64_t tests_fp32;       /* float32 pair evaluations */
  int64_t band_retests;     /* float32 evaluations re-tested in float64 */
  int64_t asym_pairs;       /* core pairs that are neighbours in one direction only
                               (the box test and the distance test disagree at the
                               last bit; their merges are replayed in order) */
  int64_t grid_cells;       /* occupancy-table entries: cells of cell tables, rows of
                               row tables (a hashed grid has none) */
  int32_t precision_used;   /* gd_precision actually run */
  int32_t key_bits;         /* radix-sort key width */
  int32_t launches;         /* kernel launches of the last pipeline run */
  int32_t reserved;
  double ms_index;          /* device time: bbox, keys, sort, cell table */
  double ms_core;           /* device time: core flags */
  double ms_union;          /* device time: union-find */
  double ms_label;          /* device time: cluster ids, borders, output order */
  double ms_total;          /* device time of the whole pipeline (without host copies) */
  double ms_h2d;            /* host->device copy of the points (0 if on device) */
  double ms_d2h;            /* device->host copy of the labels (0 if on device) */
} gd_stats;

/* ---- context ------------------------------------------------------------ */
gd_status gd_ctx_create(int32_t device, gd_ctx** out);
void gd_ctx_destroy(gd_ctx* ctx);
/* stream: a cudaStream_t of the context's device; NULL restores the context's own */
gd_status gd_ctx_set_stream(gd_ctx* ctx, void* stream);
gd_status gd_ctx_set_precision(gd_ctx* ctx, int32_t precision);
/* grid cell side = eps * mult; 0 restores the defaults: 0.5*(1+2^-16) in 2D,
   the largest allowed, (1/sqrt(3))*(1-2^-20), in 3D.
   Allowed range: (0.5, 1/sqrt(dim)) -- cells stay smaller than eps/sqrt(dim) so
   a cell's points are mutual neighbours, and larger than eps/2 so neighbours
   stay within +-2 cells. */
gd_status gd_ctx_set_cell_mult(gd_ctx* ctx, double mult);
/* Separate multipliers for 2D (range (0.5, 1/sqrt(2))) and 3D instances
   (range (0.5, 1/sqrt(3))); 0 restores the default.  Set by the autotuner. */
gd_status gd_ctx_set_cell_mults(gd_ctx* ctx, double mult2d, double mult3d);
/* Frees the context's cached device buffers (they regrow on the next call). */
gd_status gd_ctx_trim(gd_ctx* ctx);
/* No counterpart in the reference.  With graphs enabled (the default), the
   second gd_expand on one index build captures the expand launches into a CUDA
   graph and later gd_expand calls on that index (other minpts) replay it with
   one launch.  A new index build, a tuning change or gd_ctx_trim drops it. */
gd_status gd_ctx_set_graphs(gd_ctx* ctx, int32_t enable);

/* ---- the pipeline, stage by stage ---------------------------------------- */
/* Replaces main.cu:166-338: host min/max + bin widths (main.cu:166-207), the
   per-node tree allocation (main.cu:264-305), INDEXING_STRUCTURE
   (indexing.cu:54-118), thrust::sort_by_key (main.cu:332) and
   INDEXING_ADJUSTMENT (indexing.cu:23-51).  Builds the eps-cell grid of the
   points on the device; the points must stay valid until gd_expand returns. */
gd_status gd_index_build(gd_ctx* ctx, const gd_points* pts, double eps);

/* Replaces the expansion loop main.cu:369-403: MonitorSeedPoints
   (dbscan.cu:25-187), the DBSCAN kernel (dbscan.cu:254-387) and
   MarkAsCandidate (dbscan.cu:189-222).  Core flags, device union-find over
   core-core links, cluster numbering and border assignment, all on the GPU. */
gd_status gd_expand(gd_ctx* ctx, int32_t minpts);

/* Replaces GetDbscanResult (dbscan.cu:225-251).  Writes per-point labels in the
   caller's point order (host or device memory as on_device says), optional
   per-point core flags (is_core may be NULL), and the counts the reference
   prints (main.cu:423-424).  cluster_count / noise_count may be NULL. */
gd_status gd_get_result(gd_ctx* ctx, int32_t* labels, uint8_t* is_core, int32_t on_device,
                        int64_t* cluster_count, int64_t* noise_count);

/* The whole pipeline in one call (main.cu:35-459 without the CSV import):
   labels has pts->n entries in the same memory space as pts->coords.
   stats may be NULL. */
gd_status gd_dbscan(gd_ctx* ctx, const gd_points* pts, double eps, int32_t minpts,
                    int32_t* labels, gd_stats* stats);

/* Statistics of the last gd_expand / gd_dbscan on this context. */
gd_status gd_get_stats(gd_ctx* ctx, gd_stats* stats);

/* ---- many independent instances in one run ------------------------------ */
typedef struct gd_instance {
  int64_t n;        /* points of this instance */
  int32_t dim;      /* 2 or 3 */
  int32_t minpts;
  double eps;
} gd_instance;

/* No counterpart in the reference (which clusters one data set per program
   run, main.cu:35-459).  Clusters `count` independent instances, each with its
   own eps, minpts and dimension, in one pass of the pipeline: one sort, one
   cell list and one launch per phase for all of them.  coords holds the
   instances back to back, each row-major [n][dim], in the given order (host or
   device memory per on_device); labels receives one label per point in the same
   order, cluster ids restarting at 0 in every instance (NOISE = -2).
   cluster_counts (host, count entries) and stats may be NULL.  Every
   instance's labels equal those of gd_dbscan on that instance alone. */
gd_status gd_batch_dbscan(gd_ctx* ctx, int32_t count, const gd_instance* inst,
                          const double* coords, int32_t on_device, int32_t* labels,
                          int64_t* cluster_counts, gd_stats* stats);

/* ---- tuning --------------------------------------------------------------- */
/* No counterpart in the reference (whose launch shape and partition count are
   compile-time constants, common.h:10-25).  Parameters that change speed but
   never labels: the cell side as a multiple of eps per dimension (see
   gd_ctx_set_cell_mults) and the pair tests one thread spends on a core
   count, a link search and a border search before the work goes to a warp. */
typedef struct gd_tuning {
  double mult2d;          /* (0.5, 1/sqrt(2)); 0 = default */
  double mult3d;          /* (0.5, 1/sqrt(3)); 0 = default */
  int32_t core_tests;     /* 0..65536; defaults 256, 48, 160 */
  int32_t link_tests;
  int32_t border_tests;
  int32_t reserved;       /* 0 */
} gd_tuning;

gd_status gd_ctx_set_tuning(gd_ctx* ctx, const gd_tuning* t);
gd_status gd_ctx_get_tuning(gd_ctx* ctx, gd_tuning* t);
/* Autotuner: clusters the given sample (same arguments as gd_batch_dbscan,
   labels discarded) under candidate tunings, coordinate by coordinate (2D cell
   multiplier if 2D instances are present, 3D multiplier if 3D ones are, then
   the three test budgets scaled together), keeps the one with the smallest
   device time (best of `repeats` runs each, CUDA events), sets it on the
   context and returns it (best and best_ms may be NULL). */
gd_status gd_autotune(gd_ctx* ctx, int32_t count, const gd_instance* inst, const double* coords,
                      int32_t on_device, int32_t repeats, gd_tuning* best, double* best_ms);

/* ---- request server with continuous batching ---------------------------- */
/* No counterpart in the reference.  A server queues clustering requests (one
   instance each, host buffers) and runs them on `workers` threads, each with
   its own context and CUDA stream.  A free worker takes every queued request
   it may admit, first in first out, up to max_batch requests while the
   estimated device memory of all requests in flight stays within
   hbm_budget_bytes (a request larger than the budget runs alone), and
   clusters them together with gd_batch_dbscan.  Each request's labels equal
   gd_dbscan's on that request alone. */
typedef struct gd_server gd_server;

typedef struct gd_server_config {
  int32_t device;
  int32_t workers;          /* 1..16 */
  int32_t max_batch;        /* requests per batch, >= 1 */
  int32_t precision;        /* gd_precision */
  int64_t hbm_budget_bytes; /* admission limit for requests in flight */
} gd_server_config;

typedef struct gd_request_info {
  int64_t n_clusters;
  int32_t status;     /* gd_status of the batch that ran the request */
  int32_t batch_size; /* requests in that batch */
  double submit_ms;   /* times since the server was created */
  double start_ms;
  double done_ms;
} gd_request_info;

typedef struct gd_server_stats {
  int64_t submitted;
  int64_t completed;
  int64_t failed;
  int64_t batches;
  int64_t points;
  int64_t max_batch_seen;
  int64_t queued;
  int64_t inflight_bytes;
} gd_server_stats;

gd_status gd_server_create(const gd_server_config* cfg, gd_server** out);
/* Finishes every queued request, then stops the workers. */
void gd_server_destroy(gd_server* srv);
/* coords (n x dim float64, host) must stay valid and labels (n int32, host)
   unread until gd_server_wait returns for the request. */
gd_status gd_server_submit(gd_server* srv, const gd_instance* inst, const double* coords,
                           int32_t* labels, int64_t* request_id);
/* Waits for a request (timeout_ms < 0: no limit) and forgets it; returns the
   request's status, or GD_ETIMEOUT while it is unfinished.  info may be NULL. */
gd_status gd_server_wait(gd_server* srv, int64_t request_id, double timeout_ms,
                         gd_request_info* info);
gd_status gd_server_get_stats(gd_server* srv, gd_server_stats* stats);

/* ---- exact DBSCAN without any memory allocation ------------------------ */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
   or cudaFree: control and real-time loops that reserve all their device
   memory at start-up (an allocation can block for milliseconds, and cudaFree
   waits for the whole device), and plug-ins hosted by a process whose memory
   manager owns the GPU's memory and forbids allocations behind its back.
   Same labels as gd_dbscan, for up to GD_NOALLOC_MAX_POINTS points; larger n
   is rejected with GD_ERANGE.  coords_dev (n x dim float64) and labels_dev
   (n int32) are device pointers on the current device; stream may be NULL
   (default stream).  All scratch is one fixed static device array of about
   5 MiB that every GPU which loads the library keeps until the process exits;
   nothing is allocated or freed.  The first call in a CUDA context of a device
   does a one-time set-up (it looks up that array's device address); make that
   first call before any stream capture begins.  The call synchronises its
   stream twice: in the middle, to read the grid layout back to the host, and
   at the end.  Calls share the array and it keeps the last call's contents;
   calls that overlap on the GPU race and must be serialised by the caller.
   labels_dev is undefined when the call fails.  n_clusters may be NULL. */
#define GD_NOALLOC_MAX_POINTS 32768
gd_status gd_dbscan_noalloc(const double* coords_dev, int64_t n, int32_t dim, double eps,
                            int32_t minpts, int32_t precision, int32_t* labels_dev,
                            int64_t* n_clusters, void* stream);

/* ---- dataset files ------------------------------------------------------- */
/* Replaces ImportDataset (main.cu:469-498): reads a headerless CSV with dim
   comma-separated values per line (max_points <= 0: no limit; the reference
   stops at DATASET_COUNT).  A file ending in ".f64" is read as raw float64
   row-major data instead.  *out is allocated here; release with gd_free. */
gd_status gd_import_dataset(const char* path, int32_t dim, int64_t max_points, double** out,
                            int64_t* n);
/* Writes one label per line (the per-point form of dbscan.cu:242-247). */
gd_status gd_write_labels(const char* path, const int32_t* labels, int64_t n);
void gd_free(void* p);

/* ---- label-quality report ---------------------------------------------- */
/* Replaces the reference's cluster check (test-results/cluster-check.cpp,
   DetermineErrorTwoClusterResults, lines 41-199): how far labelling b of n
   points is from labelling a.  Labels equal to `noise` are noise (the
   reference's files use 0; this library's labels use GD_NOISE); any other
   value is a cluster id.  Per point: 0 when noise in exactly one labelling,
   1 when noise in both, else the Jaccard index of its two clusters.  Host code
   only (no GPU needed).  n == 0 gives score 1. */
typedef struct gd_label_quality {
  double score;          /* mean per-point score ("Final Error metric") */
  double mismatch_loss;  /* sum of (1 - score) over points clustered in both, / n */
  int64_t noise_mismatch;  /* noise in exactly one labelling */
  int64_t noise_agree;     /* noise in both */
  int64_t clusters_a;      /* distinct non-noise labels in a */
  int64_t clusters_b;      /* distinct non-noise labels in b */
  int64_t n;
} gd_label_quality;
gd_status gd_label_quality_compare(const int32_t* a, const int32_t* b, int64_t n, int32_t noise,
                                   gd_label_quality* out);

/* ---- errors -------------------------------------------------------------- */
const char* gd_status_string(gd_status s);
/* Message of the last failure on the calling thread ("" if none). */
const char* gd_last_error(void);
int32_t gd_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GBDBSCAN_H */
