// gd_api.cu -- the C ABI (include/gbdbscan.h): contexts, device memory, and the
// order in which the kernels of gd_pipeline.cu run.
//
// A run clusters K >= 1 instances (gd_index_build/gd_dbscan: K = 1;
// gd_batch_dbscan: K = count).  Stage order on the context's stream; the only
// host round-trip inside a run is one read of the 64-byte run layout, which
// sizes the key width, the cell tables and the hash:
//   build:  [H2D] per-instance bbox -> grids -> layout -> (read layout) -> keys
//           -> radix sort -> gather (sorted SoA f64 [+ centred f32]) -> cell runs
//           -> dense cell tables (counts + exclusive scan) / hash of occupied cells
//   expand: core flags -> union-find (near pass, far pass, compress, merge
//           replay) -> root marks -> scan (cluster numbers) -> labels -> borders
//   finish: scatter labels/core flags to caller order -> [D2H]
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gbdbscan.h"
#include "gd_launch.h"

namespace {

thread_local std::string g_err;

gd_status fail(gd_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

gd_status cuda_fail(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return fail(GD_ENOMEM, std::string(what) + ": " + cudaGetErrorString(e));
  }
  return fail(GD_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define GD_CUDA(call, what)                            \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

#define GD_TRY(expr)            \
  do {                          \
    gd_status s_ = (expr);      \
    if (s_ != GD_OK) return s_; \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

constexpr double kDefaultCellMult = 0.5 * (1.0 + 1.0 / 65536.0);
// pair tests one thread spends before handing its work to a warp
constexpr int kDefaultCoreTests = 256, kDefaultLinkTests = 48, kDefaultBorderTests = 160;
constexpr int kMaxTests = 65536;
// A grid takes a cell table (one occupancy bit, one core bit and one prefix bit
// per cell) when it has at most this many cells per point (or 2^26 cells for a
// single instance, 4096 per instance in a batch).
constexpr uint64_t kCellsPerPoint = 64;
// largest multipliers allowed: cell diagonal below eps (1 - 2^-20)
constexpr double kMaxCellMult2 = 0.70710678118654752 * (1.0 - 1.0 / 1048576.0);
constexpr double kMaxCellMult3 = 0.57735026918962576 * (1.0 - 1.0 / 1048576.0);
// default multipliers: the smallest cells in 2D (larger 2D cells measured
// slower: more float64 tests per walk), the largest in 3D (C3: 6.84 -> 6.33 ms,
// 27-bit keys and three sort passes instead of four, fewer link searches)
constexpr double kDefaultCellMult2 = kDefaultCellMult;
constexpr double kDefaultCellMult3 = kMaxCellMult3;

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

namespace gdio {
void set_error(const std::string& m) { g_err = m; }
}  // namespace gdio

struct gd_ctx {
  int device = 0;
  int sms = 152;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  int precision = GD_PREC_FP64;
  double mult2 = kDefaultCellMult2, mult3 = kDefaultCellMult3;
  int tn_core = kDefaultCoreTests, tn_link = kDefaultLinkTests, tn_border = kDefaultBorderTests;

  DevBuf coords, inst, chunks, Pv, Bi, bbox, keys0, keys1, vals0, vals1, X, Xf, table, occ, cellz,
      hkeys, hvals, reps, bits, core, cellcore, cellmin, parent, cellcid, lab, asym,
      hvcell, hvmask, out, coreout, sorttemp, scantemp, small, kcount;

  // the current run
  int stage = 0;  // 0: nothing, 1: indexed, 2: expanded
  int K = 0;
  int64_t n = 0;
  int dims = 0;   // bit 0: 2D instances present, bit 1: 3D
  bool f32 = false, key64 = false, xf = false;
  gd::BatchInfo bi{};
  std::vector<gd::InstDesc> hdesc;
  std::vector<gd::Chunk> hchunk;
  const double* coords_ptr = nullptr;  // the run's points on the device
  void* skeys = nullptr;
  uint32_t* sids = nullptr;
  uint32_t hmask = 0;
  cudaEvent_t ev[8] = {};
  // CUDA graph of the expand launches, captured on the second gd_expand of one
  // index build and replayed by later ones (minpts sweeps)
  bool graphs = true;
  cudaGraphExec_t xgraph = nullptr;
  int expands_on_index = 0;
  void drop_graph() {
    if (xgraph) cudaGraphExecDestroy(xgraph);
    xgraph = nullptr;
    expands_on_index = 0;
  }
  gd_stats st{};
  int launches = 0;         // kernels of the last index build
  int expand_launches = 0;  // kernels of the expand stage (the captured graph holds as many)

  gd_status ensure(DevBuf& b, size_t bytes, const char* what) {
    bytes = up256(bytes ? bytes : 1);
    if (b.bytes >= bytes) return GD_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
      b.p = nullptr;
      return cuda_fail(e, what);
    }
    b.bytes = bytes;
    return GD_OK;
  }

  // ensure() for temp memory that must be zero when first used (the scan and
  // sort state): cleared on the stream whenever it is (re)allocated
  gd_status ensure_zeroed(DevBuf& b, size_t bytes, const char* what) {
    void* before = b.p;
    const size_t had = b.bytes;
    GD_TRY(ensure(b, bytes, what));
    if (b.p != before || b.bytes != had) GD_CUDA(cudaMemsetAsync(b.p, 0, b.bytes, stream), what);
    return GD_OK;
  }

  void free_all(bool keep_small) {
    DevBuf* a[] = {&coords, &inst,   &chunks,   &Pv,      &Bi,     &bbox,     &keys0,
                   &keys1,  &vals0,  &vals1,    &X,       &Xf,     &table,    &occ, &cellz, &hkeys,
                   &hvals,  &reps,   &bits,     &core,    &cellcore, &cellmin,
                   &parent, &cellcid,  &lab,     &asym,   &hvcell,   &hvmask,
                   &out,    &coreout, &sorttemp, &scantemp, &small, &kcount};
    for (DevBuf* b : a) {
      if (keep_small && b == &small) continue;
      if (b->p) cudaFree(b->p);
      b->p = nullptr;
      b->bytes = 0;
    }
  }

  // small block: M | total clusters | counters
  uint32_t* dM() { return static_cast<uint32_t*>(small.p); }
  uint32_t* dK() { return reinterpret_cast<uint32_t*>(static_cast<char*>(small.p) + 4); }
  unsigned long long* dCtr() {
    return reinterpret_cast<unsigned long long*>(static_cast<char*>(small.p) + 128);
  }

  gdl::Bufs bufs() {
    gdl::Bufs B;
    B.coords = coords_ptr;
    B.inst = static_cast<const gd::InstDesc*>(inst.p);
    B.chunks = static_cast<const gd::Chunk*>(chunks.p);
    B.Pv = static_cast<gd::DevParams*>(Pv.p);
    B.Bi = static_cast<gd::BatchInfo*>(Bi.p);
    B.bbox = static_cast<long long*>(bbox.p);
    B.keys = skeys;
    B.ids = sids;
    // the sort's other id and key buffers are free after the sort
    B.blist = static_cast<uint32_t*>(sids == vals0.p ? vals1.p : vals0.p);
    B.reps = static_cast<int*>(reps.p);
    if (bits.p) gdl::set_bits(B, static_cast<uint32_t*>(bits.p), n);
    B.K = dK();
    B.start = static_cast<uint32_t*>(table.p);
    B.occ = static_cast<uint32_t*>(occ.p);
    B.cellz = static_cast<uint32_t*>(cellz.p);
    if (bi.occ_total) {
      // one buffer: occupancy | core occupancy | word prefix counts
      B.occ_words = bi.occ_total / 32 + 1;
      B.cocc = B.occ + B.occ_words;
      B.wpre = B.occ + gdl::occ_wpre_offset(B.occ_words);
    }
    B.hkeys = static_cast<unsigned long long*>(hkeys.p);
    B.hvals = static_cast<uint32_t*>(hvals.p);
    B.hmask = hmask;
    B.X = static_cast<double*>(X.p);
    B.Xf = static_cast<float*>(Xf.p);
    B.core = static_cast<uint8_t*>(core.p);
    B.cellcore = static_cast<int*>(cellcore.p);
    B.cellmin = static_cast<int*>(cellmin.p);
    B.parent = static_cast<int*>(parent.p);
    B.cellcid = static_cast<int*>(cellcid.p);
    B.lab = static_cast<int*>(lab.p);
    B.asym = static_cast<int*>(asym.p);
    B.hv_cell = static_cast<int*>(hvcell.p);
    B.hv_mask = static_cast<unsigned long long*>(hvmask.p);
    B.ctr = dCtr();
    B.tn_core = tn_core;
    B.tn_link = tn_link;
    B.tn_border = tn_border;
    return B;
  }
};

namespace {

// Point runs of at most kChunkPoints points, one instance each.
void make_chunks(const std::vector<gd::InstDesc>& desc, std::vector<gd::Chunk>& out) {
  out.clear();
  for (size_t i = 0; i < desc.size(); ++i)
    for (int64_t b = 0; b < desc[i].n; b += gd::kChunkPoints) {
      gd::Chunk c;
      c.inst = (int32_t)i;
      c.pad = 0;
      c.begin = desc[i].pt_off + b;
      c.end = desc[i].pt_off + std::min<int64_t>(desc[i].n, b + gd::kChunkPoints);
      out.push_back(c);
    }
}

// Build stage of a run: ctx->hdesc (internal order, 2D instances first) and
// ctx->coords_ptr (device) are set by the caller.
gd_status build_run(gd_ctx* ctx, uint64_t dense_floor, uint64_t dense_per_point) {
  ctx->drop_graph();
  cudaStream_t s = ctx->stream;
  const int K = (int)ctx->hdesc.size();
  ctx->K = K;
  int64_t n = 0;
  for (const auto& d : ctx->hdesc) n += d.n;
  ctx->n = n;
  make_chunks(ctx->hdesc, ctx->hchunk);
  const int nch = (int)ctx->hchunk.size();
  GD_TRY(ctx->ensure(ctx->inst, K * sizeof(gd::InstDesc), "instance table"));
  GD_TRY(ctx->ensure(ctx->chunks, std::max(1, nch) * sizeof(gd::Chunk), "chunk table"));
  GD_TRY(ctx->ensure(ctx->Pv, K * sizeof(gd::DevParams), "instance parameters"));
  GD_TRY(ctx->ensure(ctx->Bi, sizeof(gd::BatchInfo), "run layout"));
  GD_TRY(ctx->ensure(ctx->bbox, K * 6 * 8, "bounding boxes"));
  GD_CUDA(cudaMemcpyAsync(ctx->inst.p, ctx->hdesc.data(), K * sizeof(gd::InstDesc),
                          cudaMemcpyHostToDevice, s), "upload instances");
  if (nch)
    GD_CUDA(cudaMemcpyAsync(ctx->chunks.p, ctx->hchunk.data(), nch * sizeof(gd::Chunk),
                            cudaMemcpyHostToDevice, s), "upload chunks");
  GD_CUDA(cudaMemsetAsync(ctx->small.p, 0, ctx->small.bytes, s), "clear counters");
  GD_CUDA(cudaMemsetAsync(ctx->Bi.p, 0, sizeof(gd::BatchInfo), s), "clear layout");
  gdl::Bufs B = ctx->bufs();
  const int grid_launches =
      gdl::grids(B, K, nch, ctx->mult2, ctx->mult3, dense_floor, dense_per_point, s);
  GD_CUDA(cudaMemcpyAsync(&ctx->bi, ctx->Bi.p, sizeof(gd::BatchInfo), cudaMemcpyDeviceToHost, s),
          "read run layout");
  GD_CUDA(cudaStreamSynchronize(s), "grid parameters");
  const gd::BatchInfo& bi = ctx->bi;
  if (bi.flags & gd::kFlagNonFinite) return fail(GD_EINVAL, "input has NaN or Inf coordinates");
  if (bi.flags & gd::kFlagGridTooLarge)
    return fail(GD_ERANGE, "eps-cell grid too large (extent/eps beyond 2^31 cells per axis, or "
                           "cell keys and instance ids beyond 62 bits)");
  ctx->key64 = bi.key64 != 0;
  // float32 filter when asked for; a single instance without a valid band
  // runs the float64 kernels (a batch keeps the filter: such instances send
  // every pair to the float64 predicate)
  ctx->f32 = ctx->precision == GD_PREC_FP32_BAND && !(K == 1 && bi.band_off);
  ctx->xf = ctx->f32 || bi.any_xf;
  ctx->dims = (bi.K2 > 0 ? 1 : 0) | (bi.K2 < K ? 2 : 0);
  const size_t kw = ctx->key64 ? 8 : 4;
  const int maxd = bi.max_dim;
  GD_TRY(ctx->ensure(ctx->keys0, n * kw, "keys"));
  GD_TRY(ctx->ensure(ctx->keys1, n * kw, "keys"));
  GD_TRY(ctx->ensure(ctx->vals0, n * 4, "ids"));
  GD_TRY(ctx->ensure(ctx->vals1, n * 4, "ids"));
  GD_TRY(ctx->ensure(ctx->X, (size_t)n * maxd * 8, "sorted coordinates"));
  if (ctx->xf) GD_TRY(ctx->ensure(ctx->Xf, (size_t)n * maxd * 4, "f32 coordinates"));
  const uint64_t W = bi.occ_total ? bi.occ_total / 32 + 1 : 0;
  GD_TRY(ctx->ensure(ctx->table, std::max<uint64_t>(bi.start_total, 1) * 4, "row tables"));
  if (W) GD_TRY(ctx->ensure(ctx->occ, gdl::occ_buffer_words(W) * 4, "cell occupancy"));
  uint64_t hcap = 1024;
  if (bi.any_sparse) {
    while (hcap < 2 * (uint64_t)n) hcap <<= 1;
    GD_TRY(ctx->ensure(ctx->hkeys, hcap * 8, "row hash keys"));
    GD_TRY(ctx->ensure(ctx->hvals, hcap * 8, "row hash values"));
  }
  ctx->hmask = (uint32_t)(hcap - 1);
  GD_TRY(ctx->ensure(ctx->reps, (n + 1) * 4, "cell reps"));
  GD_TRY(ctx->ensure(ctx->cellz, n * 4, "cell coordinates"));
  GD_TRY(ctx->ensure(ctx->bits, gdl::bit_layout(n).words * 4, "bit masks"));
  GD_TRY(ctx->ensure_zeroed(ctx->sorttemp, gdprim::sort_temp_bytes(n), "sort temp"));
  size_t sc = std::max({gdprim::scan_temp_bytes(n + 1),
                        gdprim::scan_temp_bytes((int64_t)bi.start_total),
                        gdprim::scan_temp_bytes((int64_t)W)});
  GD_TRY(ctx->ensure_zeroed(ctx->scantemp, sc, "scan temp"));
  const int key_bits = bi.LB + bi.IB;
  int r;
  uint32_t* vb[2] = {static_cast<uint32_t*>(ctx->vals0.p), static_cast<uint32_t*>(ctx->vals1.p)};
  B = ctx->bufs();
  int L = grid_launches + gdl::keys(B, ctx->key64, nch, ctx->keys0.p, s);
  if (ctx->key64) {
    using U64 = unsigned long long;
    U64* kb[2] = {static_cast<U64*>(ctx->keys0.p), static_cast<U64*>(ctx->keys1.p)};
    r = gdprim::radix_sort_pairs<U64>(kb, vb, n, key_bits, true, ctx->sorttemp.p, s,
                                        ctx->dCtr() + gd::kCtrWaitTimeouts);
    ctx->skeys = kb[r];
  } else {
    uint32_t* kb[2] = {static_cast<uint32_t*>(ctx->keys0.p), static_cast<uint32_t*>(ctx->keys1.p)};
    r = gdprim::radix_sort_pairs<uint32_t>(kb, vb, n, key_bits, true, ctx->sorttemp.p, s,
                                        ctx->dCtr() + gd::kCtrWaitTimeouts);
    ctx->skeys = kb[r];
  }
  L += gdprim::sort_launches(n, key_bits);
  ctx->sids = vb[r];
  B = ctx->bufs();
  L += gdl::gather(B, ctx->key64, n, ctx->xf, K == 1, ctx->sms, s);
  L += gdl::runs(B, ctx->key64, n, ctx->dims == 3, ctx->sms, ctx->scantemp.p, s);
  // occupancy bits, row-table starts, occupancy ranks
  GD_CUDA(cudaMemsetAsync(ctx->table.p, 0, bi.start_total * 4, s), "clear row tables");
  if (W) GD_CUDA(cudaMemsetAsync(ctx->occ.p, 0, W * 4, s), "clear occupancy");
  L += gdl::cell_counts(B, ctx->key64, n, ctx->sms, s);
  L += gdl::start_fill(B, ctx->K, s);
  gdprim::exclusive_scan_u32(B.start, B.start, (int64_t)bi.start_total, ctx->scantemp.p, nullptr,
                             s, ctx->dCtr() + gd::kCtrWaitTimeouts);
  L += gdprim::scan_launches((int64_t)bi.start_total);
  L += gdl::occ_rank(B, ctx->K, ctx->scantemp.p, s);
  if (bi.any_sparse) {
    GD_CUDA(cudaMemsetAsync(ctx->hkeys.p, 0xff, hcap * 8, s), "clear row hash");
    L += gdl::hash_insert(B, ctx->key64, n, ctx->sms, s);
  }
  GD_CUDA(cudaGetLastError(), "index build launch");
  ctx->launches = L;
  ctx->st.grid_cells = (int64_t)bi.occ_total;
  ctx->st.key_bits = key_bits;
  ctx->stage = 1;
  return GD_OK;
}

// The expand launches (no allocation, no host synchronisation, so they can be
// captured).  Returns the first error; never leaves early.
cudaError_t launch_expand(gd_ctx* ctx, bool capturing) {
  cudaStream_t s = ctx->stream;
  const int64_t n = ctx->n;
  const unsigned evf = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  cudaError_t e = cudaSuccess;
  auto keep = [&](cudaError_t r) { if (e == cudaSuccess && r != cudaSuccess) e = r; };
  // counters of this stage (the build's cell counts and 2D/3D split stay)
  keep(cudaMemsetAsync(ctx->dCtr() + gd::kCtrTests64, 0,
                       (gd::kCtrHeavyBorder - gd::kCtrTests64 + 1) * 8, s));
  gdl::Bufs B = ctx->bufs();
  keep(cudaEventRecordWithFlags(ctx->ev[3], s, evf));
  int L = gdl::core(B, n, ctx->dims, ctx->f32, ctx->key64, ctx->K == 1, ctx->sms,
                    ctx->scantemp.p, s);
  keep(cudaEventRecordWithFlags(ctx->ev[4], s, evf));
  L += gdl::unite(B, n, ctx->dims, ctx->f32, ctx->key64, ctx->sms, ctx->scantemp.p, s);
  keep(cudaEventRecordWithFlags(ctx->ev[5], s, evf));
  L += gdl::roots(B, ctx->key64, n, ctx->sms, ctx->scantemp.p, s);
  L += gdl::label(B, n, ctx->sms, ctx->scantemp.p, s);
  L += gdl::border(B, n, ctx->dims, ctx->f32, ctx->key64, ctx->sms, s);
  keep(cudaGetLastError());
  ctx->expand_launches = L;
  return e;
}

gd_status expand_run(gd_ctx* ctx) {
  cudaStream_t s = ctx->stream;
  const int64_t n = ctx->n;
  GD_TRY(ctx->ensure(ctx->core, n, "core flags"));
  GD_TRY(ctx->ensure(ctx->cellcore, n * 4, "cell core counts"));
  GD_TRY(ctx->ensure(ctx->cellmin, n * 4, "cell min index"));
  GD_TRY(ctx->ensure(ctx->parent, n * 4, "union-find parents"));
  GD_TRY(ctx->ensure(ctx->cellcid, n * 4, "cell cluster ids"));
  GD_TRY(ctx->ensure(ctx->lab, n * 4, "labels"));
  GD_TRY(ctx->ensure(ctx->asym, gd::kAsymCap * 8, "one-directional links"));
  GD_TRY(ctx->ensure(ctx->hvcell, n * 4, "heavy-work list"));
  GD_TRY(ctx->ensure(ctx->hvmask, n * 8, "heavy-work masks"));
  GD_TRY(ctx->ensure_zeroed(ctx->scantemp,
                            std::max(gdprim::scan_temp_bytes(n + 1), ctx->scantemp.bytes),
                            "scan temp"));
  ctx->stage = 2;
  if (ctx->graphs && ctx->xgraph) {
    GD_CUDA(cudaGraphLaunch(ctx->xgraph, s), "expand graph launch");
    return GD_OK;
  }
  // capture on the second expand of this index build: a first one is often
  // the only one (gd_dbscan), and capturing costs more than launching once
  bool capture = ctx->graphs && ctx->expands_on_index >= 1;
  ++ctx->expands_on_index;
  if (capture && cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    capture = false;
  }
  cudaError_t e = launch_expand(ctx, capture);
  if (!capture) {
    if (e != cudaSuccess) return cuda_fail(e, "expand launch");
    return GD_OK;
  }
  cudaGraph_t g = nullptr;
  cudaError_t ec = cudaStreamEndCapture(s, &g);
  if (e == cudaSuccess && ec == cudaSuccess && g) ec = cudaGraphInstantiate(&ctx->xgraph, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess || ec != cudaSuccess) {
    // nothing captured ran: give up graphs for this context and launch directly
    cudaGetLastError();
    ctx->xgraph = nullptr;
    ctx->graphs = false;
    e = launch_expand(ctx, false);
    if (e != cudaSuccess) return cuda_fail(e, "expand launch");
    return GD_OK;
  }
  GD_CUDA(cudaGraphLaunch(ctx->xgraph, s), "expand graph launch");
  return GD_OK;
}

// Scatter labels (and core flags) to the caller's point order, copy them out,
// read the counters into ctx->st.
// Scatter labels (and core flags) to the caller's order, copy them out, read the
// counters, all behind one stream synchronisation.  A batch also passes its
// per-instance cluster-count array (kc, kc_count entries in sorted-instance
// order), filled before that same synchronisation.
gd_status finish_run(gd_ctx* ctx, int32_t* labels, uint8_t* is_core, int32_t on_device,
                     int64_t* kc = nullptr, int kc_count = 0) {
  cudaStream_t s = ctx->stream;
  const int64_t n = ctx->n;
  gd_stats& S = ctx->st;
  int* out = reinterpret_cast<int*>(labels);
  uint8_t* cout = is_core;
  if (!on_device) {
    GD_TRY(ctx->ensure(ctx->out, n * 4, "label output"));
    out = static_cast<int*>(ctx->out.p);
    if (is_core) {
      GD_TRY(ctx->ensure(ctx->coreout, n, "core output"));
      cout = static_cast<uint8_t*>(ctx->coreout.p);
    }
  }
  GD_CUDA(cudaMemsetAsync(ctx->dCtr() + gd::kCtrCore, 0, 2 * 8, s), "clear counters");
  gdl::Bufs B = ctx->bufs();
  int fin = gdl::scatter_labels(B, n, out, cout, ctx->sms, s);
  cudaEventRecord(ctx->ev[6], s);
  if (!on_device) {
    GD_CUDA(cudaMemcpyAsync(labels, out, n * 4, cudaMemcpyDeviceToHost, s), "copy labels");
    if (is_core)
      GD_CUDA(cudaMemcpyAsync(is_core, cout, n, cudaMemcpyDeviceToHost, s), "copy core flags");
  }
  if (kc && kc_count > 0) {
    GD_TRY(ctx->ensure(ctx->kcount, (int64_t)kc_count * 8, "cluster counts"));
    fin += gdl::cluster_counts(ctx->bufs(), kc_count, static_cast<int64_t*>(ctx->kcount.p), s);
    GD_CUDA(cudaMemcpyAsync(kc, ctx->kcount.p, (size_t)kc_count * 8, cudaMemcpyDeviceToHost, s),
            "copy cluster counts");
  }
  cudaEventRecord(ctx->ev[7], s);
  unsigned long long ctr[gd::kCtrCount];
  uint32_t K = 0;
  GD_CUDA(cudaMemcpyAsync(ctr, ctx->dCtr(), sizeof ctr, cudaMemcpyDeviceToHost, s), "counters");
  GD_CUDA(cudaMemcpyAsync(&K, ctx->dK(), 4, cudaMemcpyDeviceToHost, s), "cluster count");
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "DBSCAN pipeline");
  S.n_points = n;
  S.n_clusters = K;
  S.n_noise = (int64_t)ctr[gd::kCtrNoise];
  S.n_core = (int64_t)ctr[gd::kCtrCore];
  S.n_border = n - S.n_noise - S.n_core;
  S.n_cells = (int64_t)ctr[gd::kCtrCells];
  S.n_dense_cells = (int64_t)ctr[gd::kCtrDenseCells];
  S.tests_fp64 = (int64_t)ctr[gd::kCtrTests64];
  S.tests_fp32 = (int64_t)ctr[gd::kCtrTests32];
  S.band_retests = (int64_t)ctr[gd::kCtrBand];
  S.asym_pairs = (int64_t)ctr[gd::kCtrAsym];
  S.precision_used = ctx->f32 ? GD_PREC_FP32_BAND : GD_PREC_FP64;
  S.launches = ctx->launches + ctx->expand_launches + fin;
  if (ctr[gd::kCtrWaitTimeouts]) {
    // start the scan and sort state afresh for the next run
    if (ctx->sorttemp.p) cudaMemsetAsync(ctx->sorttemp.p, 0, ctx->sorttemp.bytes, s);
    if (ctx->scantemp.p) cudaMemsetAsync(ctx->scantemp.p, 0, ctx->scantemp.bytes, s);
    cudaStreamSynchronize(s);
    ctx->stage = 1;
    return fail(GD_ECUDA, "a scan or sort look-back wait gave up (results discarded)");
  }
  if (ctr[gd::kCtrAsymEdges] > (unsigned long long)gd::kAsymCap) {
    ctx->stage = 1;
    return fail(GD_ERANGE, "more one-directional core neighbour pairs than the merge replay "
                           "holds (2048)");
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  S.ms_h2d = ms;
  cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
  S.ms_index = ms;
  cudaEventElapsedTime(&ms, ctx->ev[3], ctx->ev[4]);
  S.ms_core = ms;
  cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
  S.ms_union = ms;
  cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]);
  S.ms_label = ms;
  cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]);
  S.ms_d2h = ms;
  S.ms_total = S.ms_index + S.ms_core + S.ms_union + S.ms_label;
  return GD_OK;
}

// Points of a run on the device: the caller's device pointer, or a copy of
// the caller's host buffer.
gd_status stage_points(gd_ctx* ctx, const double* coords, int64_t doubles, int32_t on_device) {
  if (on_device || doubles == 0) {
    ctx->coords_ptr = coords;
    return GD_OK;
  }
  GD_TRY(ctx->ensure(ctx->coords, doubles * 8, "points"));
  GD_CUDA(cudaMemcpyAsync(ctx->coords.p, coords, doubles * 8, cudaMemcpyHostToDevice,
                          ctx->stream), "copy points to device");
  ctx->coords_ptr = static_cast<const double*>(ctx->coords.p);
  return GD_OK;
}

}  // namespace

extern "C" {

int32_t gd_abi_version(void) { return GD_ABI_VERSION; }

const char* gd_last_error(void) { return g_err.c_str(); }

const char* gd_status_string(gd_status s) {
  switch (s) {
    case GD_OK: return "ok";
    case GD_EINVAL: return "invalid argument";
    case GD_ENOMEM: return "out of memory";
    case GD_ECUDA: return "CUDA error";
    case GD_ERANGE: return "grid too large";
    case GD_ETIMEOUT: return "timed out";
    case GD_EIO: return "I/O error";
    case GD_ENODEV: return "no suitable device";
    case GD_ESTATE: return "call out of order";
  }
  return "unknown status";
}

gd_status gd_ctx_create(int32_t device, gd_ctx** out) {
  if (!out) return fail(GD_EINVAL, "gd_ctx_create: out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(GD_ENODEV, "gd_ctx_create: no CUDA device available");
  }
  if (device < 0 || device >= count) return fail(GD_EINVAL, "gd_ctx_create: bad device index");
  cudaDeviceProp prop;
  GD_CUDA(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
  if (!(prop.major == 10 && prop.minor == 3))
    return fail(GD_ENODEV, std::string("gd_ctx_create: built for sm_103a, device is sm_") +
                               std::to_string(prop.major) + std::to_string(prop.minor));
  GD_CUDA(cudaSetDevice(device), "cudaSetDevice");
  gd_ctx* c = new gd_ctx();
  c->device = device;
  c->sms = prop.multiProcessorCount;
  e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaStreamCreate");
  }
  c->stream = c->own;
  for (auto& ev : c->ev) cudaEventCreate(&ev);
  gd_status s = c->ensure(c->small, 4096, "small buffer");
  if (s != GD_OK) {
    gd_ctx_destroy(c);
    return s;
  }
  *out = c;
  return GD_OK;
}

void gd_ctx_destroy(gd_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->drop_graph();
  ctx->free_all(false);
  for (auto& ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->own) cudaStreamDestroy(ctx->own);
  delete ctx;
}

gd_status gd_ctx_set_stream(gd_ctx* ctx, void* stream) {
  if (!ctx) return fail(GD_EINVAL, "NULL context");
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
  return GD_OK;
}

gd_status gd_ctx_set_precision(gd_ctx* ctx, int32_t precision) {
  if (!ctx) return fail(GD_EINVAL, "NULL context");
  if (precision != GD_PREC_FP64 && precision != GD_PREC_FP32_BAND)
    return fail(GD_EINVAL, "unknown precision mode");
  ctx->precision = precision;
  return GD_OK;
}

gd_status gd_ctx_set_cell_mult(gd_ctx* ctx, double mult) {
  return gd_ctx_set_cell_mults(ctx, mult, mult);
}

gd_status gd_ctx_set_cell_mults(gd_ctx* ctx, double mult2d, double mult3d) {
  if (!ctx) return fail(GD_EINVAL, "NULL context");
  if (mult2d != 0.0 && !(mult2d > 0.5 && mult2d <= kMaxCellMult2))
    return fail(GD_EINVAL, "2D cell multiplier must lie in (0.5, 1/sqrt(2)) or be 0");
  if (mult3d != 0.0 && !(mult3d > 0.5 && mult3d <= kMaxCellMult3))
    return fail(GD_EINVAL, "3D cell multiplier must lie in (0.5, 1/sqrt(3)) or be 0");
  ctx->mult2 = mult2d != 0.0 ? mult2d : kDefaultCellMult2;
  ctx->mult3 = mult3d != 0.0 ? mult3d : kDefaultCellMult3;
  return GD_OK;
}

gd_status gd_ctx_set_graphs(gd_ctx* ctx, int32_t enable) {
  if (!ctx) return fail(GD_EINVAL, "gd_ctx_set_graphs: NULL context");
  ctx->drop_graph();
  ctx->graphs = enable != 0;
  return GD_OK;
}

gd_status gd_ctx_set_tuning(gd_ctx* ctx, const gd_tuning* t) {
  if (!ctx || !t) return fail(GD_EINVAL, "gd_ctx_set_tuning: NULL argument");
  auto ok = [](int32_t v) { return v >= 0 && v <= kMaxTests; };
  if (!ok(t->core_tests) || !ok(t->link_tests) || !ok(t->border_tests) || t->reserved != 0)
    return fail(GD_EINVAL, "gd_ctx_set_tuning: test budgets must lie in [0, 65536], reserved 0");
  GD_TRY(gd_ctx_set_cell_mults(ctx, t->mult2d, t->mult3d));
  ctx->tn_core = t->core_tests;
  ctx->tn_link = t->link_tests;
  ctx->tn_border = t->border_tests;
  ctx->drop_graph();  // the captured launches carry the budgets
  return GD_OK;
}

gd_status gd_ctx_get_tuning(gd_ctx* ctx, gd_tuning* t) {
  if (!ctx || !t) return fail(GD_EINVAL, "gd_ctx_get_tuning: NULL argument");
  *t = gd_tuning{ctx->mult2, ctx->mult3, ctx->tn_core, ctx->tn_link, ctx->tn_border, 0};
  return GD_OK;
}

gd_status gd_autotune(gd_ctx* ctx, int32_t count, const gd_instance* inst, const double* coords,
                      int32_t on_device, int32_t repeats, gd_tuning* best, double* best_ms) {
  if (!ctx || (count > 0 && !inst)) return fail(GD_EINVAL, "gd_autotune: NULL argument");
  if (repeats < 1 || repeats > 100) return fail(GD_EINVAL, "gd_autotune: repeats must be 1..100");
  bool has2 = false, has3 = false;
  int64_t pts = 0;
  for (int i = 0; i < count; ++i) {
    has2 |= inst[i].dim == 2 && inst[i].n > 0;
    has3 |= inst[i].dim == 3 && inst[i].n > 0;
    pts += inst[i].n > 0 ? inst[i].n : 0;
  }
  gd_tuning cur;
  GD_TRY(gd_ctx_get_tuning(ctx, &cur));
  // labels go to a scratch buffer in the sample's memory space
  std::vector<int32_t> hlab;
  void* dlab = nullptr;
  if (on_device) {
    if (pts > 0) GD_CUDA(cudaMalloc(&dlab, (size_t)pts * 4), "autotune label buffer");
  } else {
    hlab.resize((size_t)std::max<int64_t>(pts, 1));
  }
  int32_t* lab = on_device ? static_cast<int32_t*>(dlab) : hlab.data();
  // device time of one tuning: best of `repeats` runs after one warm-up
  auto eval = [&](const gd_tuning& t, double& ms) -> gd_status {
    GD_TRY(gd_ctx_set_tuning(ctx, &t));
    ms = 1e300;
    for (int r = 0; r <= repeats; ++r) {
      gd_stats st;
      GD_TRY(gd_batch_dbscan(ctx, count, inst, coords, on_device, lab, nullptr, &st));
      if (r > 0) ms = std::min(ms, st.ms_total);
    }
    return GD_OK;
  };
  double cur_ms = 0;
  gd_status st = eval(cur, cur_ms);
  // coordinate descent over the multipliers, then the budgets
  const double m2c[] = {kDefaultCellMult, 0.55, 0.6, 0.65, kMaxCellMult2};
  const double m3c[] = {kDefaultCellMult, 0.53, 0.555, kMaxCellMult3};
  const double scale[] = {0.25, 0.5, 2.0, 4.0};
  for (int axis = 0; axis < 3 && st == GD_OK; ++axis) {
    if ((axis == 0 && !has2) || (axis == 1 && !has3)) continue;
    const int nc = axis == 0 ? 5 : 4;
    const gd_tuning base = cur;
    for (int c = 0; c < nc && st == GD_OK; ++c) {
      gd_tuning t = base;
      if (axis == 0) t.mult2d = m2c[c];
      else if (axis == 1) t.mult3d = m3c[c];
      else {
        auto sc = [&](int v) { return std::min(kMaxTests, std::max(1, (int)(v * scale[c]))); };
        t.core_tests = sc(base.core_tests);
        t.link_tests = sc(base.link_tests);
        t.border_tests = sc(base.border_tests);
      }
      double ms = 0;
      st = eval(t, ms);
      if (st == GD_OK && ms < cur_ms) {
        cur = t;
        cur_ms = ms;
      }
    }
  }
  if (dlab) cudaFree(dlab);
  if (st != GD_OK) return st;
  GD_TRY(gd_ctx_set_tuning(ctx, &cur));
  if (best) *best = cur;
  if (best_ms) *best_ms = cur_ms;
  return GD_OK;
}

gd_status gd_ctx_trim(gd_ctx* ctx) {
  if (!ctx) return fail(GD_EINVAL, "NULL context");
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->drop_graph();
  ctx->free_all(true);
  ctx->stage = 0;
  return GD_OK;
}

gd_status gd_index_build(gd_ctx* ctx, const gd_points* pts, double eps) {
  if (!ctx || !pts) return fail(GD_EINVAL, "gd_index_build: NULL argument");
  if (pts->n < 0 || (pts->dim != 2 && pts->dim != 3))
    return fail(GD_EINVAL, "gd_index_build: n must be >= 0 and dim 2 or 3");
  if (!(eps > 0) || !std::isfinite(eps))
    return fail(GD_EINVAL, "gd_index_build: eps must be positive and finite");
  if (pts->n > 0 && !pts->coords) return fail(GD_EINVAL, "gd_index_build: coords is NULL");
  if (pts->n >= (int64_t)INT32_MAX) return fail(GD_EINVAL, "gd_index_build: n must be < 2^31");
  GD_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->stage = 0;
  ctx->st = gd_stats{};
  ctx->st.n_points = pts->n;
  ctx->launches = 0;
  cudaEventRecord(ctx->ev[0], ctx->stream);
  GD_TRY(stage_points(ctx, pts->coords, pts->n * pts->dim, pts->on_device));
  cudaEventRecord(ctx->ev[1], ctx->stream);
  ctx->hdesc.assign(1, gd::InstDesc{0, pts->n, 0, eps, pts->dim, 1});
  if (pts->n == 0) {
    ctx->K = 1;
    ctx->n = 0;
    ctx->stage = 1;
    return GD_OK;
  }
  GD_TRY(build_run(ctx, (uint64_t)1 << 26, kCellsPerPoint));
  cudaEventRecord(ctx->ev[2], ctx->stream);
  return GD_OK;
}

gd_status gd_expand(gd_ctx* ctx, int32_t minpts) {
  if (!ctx) return fail(GD_EINVAL, "gd_expand: NULL context");
  if (ctx->stage < 1) return fail(GD_ESTATE, "gd_expand: call gd_index_build first");
  if (minpts < 1) return fail(GD_EINVAL, "gd_expand: minpts must be >= 1");
  GD_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (ctx->n == 0) {
    ctx->stage = 2;
    return GD_OK;
  }
  if (ctx->K == 1) {
    // minpts does not shape the grid: set it in the instance's parameters
    gd::DevParams* P0 = static_cast<gd::DevParams*>(ctx->Pv.p);
    ctx->hdesc[0].minpts = minpts;
    GD_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(P0) + offsetof(gd::DevParams, minpts),
                            &ctx->hdesc[0].minpts, sizeof(int32_t), cudaMemcpyHostToDevice,
                            ctx->stream), "write minpts");
  }
  return expand_run(ctx);
}

gd_status gd_get_result(gd_ctx* ctx, int32_t* labels, uint8_t* is_core, int32_t on_device,
                        int64_t* cluster_count, int64_t* noise_count) {
  if (!ctx) return fail(GD_EINVAL, "gd_get_result: NULL context");
  if (ctx->stage < 2) return fail(GD_ESTATE, "gd_get_result: call gd_expand first");
  GD_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (ctx->n == 0) {
    if (cluster_count) *cluster_count = 0;
    if (noise_count) *noise_count = 0;
    return GD_OK;
  }
  if (!labels) return fail(GD_EINVAL, "gd_get_result: labels is NULL");
  GD_TRY(finish_run(ctx, labels, is_core, on_device));
  if (cluster_count) *cluster_count = ctx->st.n_clusters;
  if (noise_count) *noise_count = ctx->st.n_noise;
  return GD_OK;
}

gd_status gd_dbscan(gd_ctx* ctx, const gd_points* pts, double eps, int32_t minpts,
                    int32_t* labels, gd_stats* stats) {
  if (!ctx || !pts) return fail(GD_EINVAL, "gd_dbscan: NULL argument");
  if (minpts < 1) return fail(GD_EINVAL, "gd_dbscan: minpts must be >= 1");
  GD_TRY(gd_index_build(ctx, pts, eps));
  GD_TRY(gd_expand(ctx, minpts));
  GD_TRY(gd_get_result(ctx, labels, nullptr, pts->on_device, nullptr, nullptr));
  if (stats) *stats = ctx->st;
  return GD_OK;
}

gd_status gd_batch_dbscan(gd_ctx* ctx, int32_t count, const gd_instance* inst,
                          const double* coords, int32_t on_device, int32_t* labels,
                          int64_t* cluster_counts, gd_stats* stats) {
  if (!ctx || (count > 0 && !inst)) return fail(GD_EINVAL, "gd_batch_dbscan: NULL argument");
  if (count < 0) return fail(GD_EINVAL, "gd_batch_dbscan: count must be >= 0");
  GD_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->stage = 0;
  ctx->st = gd_stats{};
  ctx->launches = 0;
  // validate; caller layout offsets; internal order puts 2D instances first
  std::vector<gd::InstDesc> user(count);
  int64_t pt = 0, co = 0;
  for (int i = 0; i < count; ++i) {
    const gd_instance& I = inst[i];
    if (I.n < 0 || (I.dim != 2 && I.dim != 3) || !(I.eps > 0) || !std::isfinite(I.eps) ||
        I.minpts < 1)
      return fail(GD_EINVAL, "gd_batch_dbscan: instance " + std::to_string(i) +
                                 " has n < 0, dim not 2/3, eps not positive and finite, or "
                                 "minpts < 1");
    user[i] = gd::InstDesc{pt, I.n, co, I.eps, I.dim, I.minpts};
    pt += I.n;
    co += I.n * I.dim;
  }
  if (pt >= (int64_t)INT32_MAX) return fail(GD_EINVAL, "gd_batch_dbscan: total points >= 2^31");
  if (pt > 0 && (!coords || !labels)) return fail(GD_EINVAL, "gd_batch_dbscan: NULL buffer");
  ctx->st.n_points = pt;
  std::vector<int> order;
  order.reserve(count);
  for (int pass = 2; pass <= 3; ++pass)
    for (int i = 0; i < count; ++i)
      if (user[i].dim == pass) order.push_back(i);
  ctx->hdesc.resize(count);
  for (int j = 0; j < count; ++j) ctx->hdesc[j] = user[order[j]];
  cudaEventRecord(ctx->ev[0], ctx->stream);
  GD_TRY(stage_points(ctx, coords, co, on_device));
  cudaEventRecord(ctx->ev[1], ctx->stream);
  if (pt == 0 || count == 0) {
    ctx->K = count;
    ctx->n = 0;
    if (cluster_counts)
      for (int i = 0; i < count; ++i) cluster_counts[i] = 0;
    if (stats) *stats = ctx->st;
    return GD_OK;
  }
  GD_TRY(build_run(ctx, 4096, kCellsPerPoint));
  cudaEventRecord(ctx->ev[2], ctx->stream);
  GD_TRY(expand_run(ctx));
  std::vector<int64_t> kc(cluster_counts ? count : 0);
  GD_TRY(finish_run(ctx, labels, nullptr, on_device, kc.data(), (int)kc.size()));
  if (cluster_counts)
    for (int j = 0; j < count; ++j) cluster_counts[order[j]] = kc[j];
  if (stats) *stats = ctx->st;
  return GD_OK;
}

gd_status gd_get_stats(gd_ctx* ctx, gd_stats* stats) {
  if (!ctx || !stats) return fail(GD_EINVAL, "gd_get_stats: NULL argument");
  *stats = ctx->st;
  return GD_OK;
}

}  // extern "C"
