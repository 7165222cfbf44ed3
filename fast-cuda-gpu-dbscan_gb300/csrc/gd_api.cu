// gd_api.cu -- the C ABI (include/gbdbscan.h): contexts, device memory, and the
// order in which the kernels of gd_pipeline.cu run for one instance.
//
// Stage order on the context's stream (no host round-trip except one 240-byte
// read of the grid parameters, which sizes the cell table):
//   gd_index_build: [H2D] bbox -> params -> (read params) -> keys -> radix sort
//                   -> gather (sorted SoA f64 [+ centred f32]) -> cell runs
//                   -> dense cell table (counts + exclusive scan)
//   gd_expand:      core flags -> union-find (near pass, far pass, compress)
//                   -> root marks -> scan (cluster ids) -> labels -> borders
//   gd_get_result:  scatter labels/core flags to caller order -> [D2H]
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

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

#define GD_CUDA(call, what)                         \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

constexpr double kDefaultCellMult = 0.5 * (1.0 + 1.0 / 65536.0);

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
  double cell_mult = 0.0;

  DevBuf pts, keys0, keys1, vals0, vals1, X, Xf, table, reps, runfl, runpos, core, cellcore,
      cellmin, parent, Fmark, cellcid, lab, out, coreout, sorttemp, scantemp, partial, small,
      asym, hkeys, hvals, hvcell, hvmask;

  // state of the current instance
  int stage = 0;  // 0: nothing, 1: indexed, 2: expanded
  int64_t n = 0;
  int dim = 2;
  double eps = 0;
  int minpts = 0;
  bool f32 = false;
  gd::DevParams hp{};
  const double* dpts = nullptr;
  void* skeys = nullptr;
  uint32_t* sids = nullptr;
  bool sparse = false;
  uint32_t hmask = 0;
  cudaEvent_t ev[8] = {};
  gd_stats st{};
  int bbox_blocks = 0;
  int launches = 0;

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

  void free_all() {
    DevBuf* all[] = {&pts, &keys0, &keys1, &vals0, &vals1, &X, &Xf, &table, &reps, &runfl,
                     &runpos, &core, &cellcore, &cellmin, &parent, &Fmark, &cellcid, &lab,
                     &out, &coreout, &sorttemp, &scantemp, &partial, &small, &asym, &hkeys,
                     &hvals, &hvcell, &hvmask};
    for (DevBuf* b : all) {
      if (b->p) cudaFree(b->p);
      b->p = nullptr;
      b->bytes = 0;
    }
  }

  // small block: params | M | K | flags | counters
  gd::DevParams* dP() { return static_cast<gd::DevParams*>(small.p); }
  uint32_t* dM() { return reinterpret_cast<uint32_t*>(static_cast<char*>(small.p) + 512); }
  uint32_t* dK() { return reinterpret_cast<uint32_t*>(static_cast<char*>(small.p) + 516); }
  int* dFlags() { return reinterpret_cast<int*>(static_cast<char*>(small.p) + 520); }
  unsigned long long* dCtr() {
    return reinterpret_cast<unsigned long long*>(static_cast<char*>(small.p) + 640);
  }

  gdl::Bufs bufs() {
    gdl::Bufs B;
    B.P = dP();
    B.keys = skeys;
    B.ids = sids;
    B.reps = static_cast<int*>(reps.p);
    B.M = dM();
    B.runfl = static_cast<uint32_t*>(runfl.p);
    B.runpos = static_cast<uint32_t*>(runpos.p);
    B.start = static_cast<uint32_t*>(table.p);
    B.hkeys = static_cast<unsigned long long*>(hkeys.p);
    B.hvals = static_cast<uint32_t*>(hvals.p);
    B.hmask = hmask;
    B.X = static_cast<double*>(X.p);
    B.Xf = static_cast<float*>(Xf.p);
    B.core = static_cast<uint8_t*>(core.p);
    B.cellcore = static_cast<int*>(cellcore.p);
    B.cellmin = static_cast<int*>(cellmin.p);
    B.parent = static_cast<int*>(parent.p);
    B.Fmark = static_cast<uint32_t*>(Fmark.p);
    B.cellcid = static_cast<int*>(cellcid.p);
    B.lab = static_cast<int*>(lab.p);
    B.asym = static_cast<int*>(asym.p);
    B.hv_cell = static_cast<int*>(hvcell.p);
    B.hv_mask = static_cast<unsigned long long*>(hvmask.p);
    B.ctr = dCtr();
    return B;
  }
};

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
  ctx->free_all();
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
  if (!ctx) return fail(GD_EINVAL, "NULL context");
  if (mult != 0.0 && !(mult > 0.5 && mult < 0.5773))
    return fail(GD_EINVAL, "cell multiplier must lie in (0.5, 1/sqrt(3)) or be 0");
  ctx->cell_mult = mult;
  return GD_OK;
}

gd_status gd_ctx_trim(gd_ctx* ctx) {
  if (!ctx) return fail(GD_EINVAL, "NULL context");
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  DevBuf keep = ctx->small;
  ctx->small = DevBuf{};
  ctx->free_all();
  ctx->small = keep;
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
  cudaStream_t s = ctx->stream;
  const int64_t n = pts->n;
  const int D = pts->dim;
  ctx->stage = 0;
  ctx->n = n;
  ctx->dim = D;
  ctx->eps = eps;
  ctx->st = gd_stats{};
  ctx->st.n_points = n;
  gd_status st;
  GD_CUDA(cudaMemsetAsync(ctx->small.p, 0, ctx->small.bytes, s), "memset");
  ctx->launches = 0;
  if (n == 0) {
    ctx->stage = 1;
    return GD_OK;
  }
  cudaEventRecord(ctx->ev[0], s);
  if (pts->on_device) {
    ctx->dpts = pts->coords;
  } else {
    if ((st = ctx->ensure(ctx->pts, (size_t)n * D * 8, "points")) != GD_OK) return st;
    GD_CUDA(cudaMemcpyAsync(ctx->pts.p, pts->coords, (size_t)n * D * 8, cudaMemcpyHostToDevice, s),
            "copy points to device");
    ctx->dpts = static_cast<const double*>(ctx->pts.p);
  }
  cudaEventRecord(ctx->ev[1], s);
  // bounding box and grid parameters
  int nb = (int)std::min<int64_t>((int64_t)ctx->sms * 4, (n + 255) / 256);
  if (nb < 1) nb = 1;
  ctx->bbox_blocks = nb;
  if ((st = ctx->ensure(ctx->partial, (size_t)nb * 6 * 8, "bbox partials")) != GD_OK) return st;
  gdl::bbox(ctx->dpts, n, D, static_cast<double*>(ctx->partial.p), nb, ctx->dFlags(), s);
  const double mult = ctx->cell_mult > 0 ? ctx->cell_mult : kDefaultCellMult;
  uint64_t max_cells = std::max<uint64_t>((uint64_t)1 << 26, (uint64_t)n * 8);
  if (max_cells > 0xfffffff0ull) max_cells = 0xfffffff0ull;
  gdl::params(static_cast<double*>(ctx->partial.p), nb, D, ctx->dP(), eps, 1, mult, max_cells,
              ctx->dFlags(), s);
  GD_CUDA(cudaMemcpyAsync(&ctx->hp, ctx->dP(), sizeof(gd::DevParams), cudaMemcpyDeviceToHost, s),
          "read grid parameters");
  GD_CUDA(cudaStreamSynchronize(s), "grid parameters");
  if (ctx->hp.flags & gd::kFlagNonFinite)
    return fail(GD_EINVAL, "gd_index_build: input has NaN or Inf coordinates");
  if (ctx->hp.flags & gd::kFlagGridTooLarge) {
    return fail(GD_ERANGE,
                "gd_index_build: eps-cell grid too large (extent/eps beyond 2^31 cells per "
                "axis or 2^62 cells in all)");
  }
  ctx->f32 = ctx->precision == GD_PREC_FP32_BAND && ctx->hp.eps2_lo32 > 0.0f;
  ctx->sparse = ctx->hp.sparse != 0;
  const uint64_t C = ctx->hp.C;
  const size_t kw = ctx->sparse ? 8 : 4;  // key width
  // buffers
  if ((st = ctx->ensure(ctx->keys0, n * kw, "keys")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->keys1, n * kw, "keys")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->vals0, n * 4, "ids")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->vals1, n * 4, "ids")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->X, (size_t)n * D * 8, "sorted coordinates")) != GD_OK) return st;
  const bool want_xf = ctx->f32 || ctx->hp.prune;  // centred float32 copy
  if (want_xf && (st = ctx->ensure(ctx->Xf, (size_t)n * D * 4, "f32 coordinates")) != GD_OK)
    return st;
  uint64_t hcap = 1024;
  if (ctx->sparse) {
    while (hcap < 2 * (uint64_t)n) hcap <<= 1;
    ctx->hmask = (uint32_t)(hcap - 1);
    if ((st = ctx->ensure(ctx->hkeys, hcap * 8, "cell hash keys")) != GD_OK) return st;
    if ((st = ctx->ensure(ctx->hvals, hcap * 4, "cell hash values")) != GD_OK) return st;
  } else {
    if ((st = ctx->ensure(ctx->table, (C + 1) * 4, "cell table")) != GD_OK) return st;
  }
  if ((st = ctx->ensure(ctx->reps, (n + 1) * 4, "cell reps")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->runfl, n * 4, "run flags")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->runpos, n * 4, "run positions")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->sorttemp, gdprim::sort_temp_bytes(n), "sort temp")) != GD_OK)
    return st;
  size_t sc = gdprim::scan_temp_bytes(n);
  if (!ctx->sparse) sc = std::max(sc, gdprim::scan_temp_bytes((int64_t)C + 1));
  if ((st = ctx->ensure(ctx->scantemp, sc, "scan temp")) != GD_OK) return st;
  // keys and sort
  int r;
  gdl::keys(ctx->dpts, n, D, ctx->sparse, ctx->dP(), ctx->keys0.p, ctx->sms, s);
  uint32_t* vb[2] = {static_cast<uint32_t*>(ctx->vals0.p), static_cast<uint32_t*>(ctx->vals1.p)};
  if (ctx->sparse) {
    using U64 = unsigned long long;
    U64* kb[2] = {static_cast<U64*>(ctx->keys0.p), static_cast<U64*>(ctx->keys1.p)};
    r = gdprim::radix_sort_pairs<U64>(kb, vb, n, ctx->hp.key_bits, true, ctx->sorttemp.p, s);
    ctx->skeys = kb[r];
  } else {
    uint32_t* kb[2] = {static_cast<uint32_t*>(ctx->keys0.p), static_cast<uint32_t*>(ctx->keys1.p)};
    r = gdprim::radix_sort_pairs<uint32_t>(kb, vb, n, ctx->hp.key_bits, true, ctx->sorttemp.p, s);
    ctx->skeys = kb[r];
  }
  ctx->sids = vb[r];
  gdl::gather(ctx->dpts, ctx->sids, n, D, want_xf, ctx->dP(), static_cast<double*>(ctx->X.p),
              static_cast<float*>(ctx->Xf.p), ctx->sms, s);
  // cell runs and the cell lookup (dense table or hash of occupied cells)
  uint32_t* fl = static_cast<uint32_t*>(ctx->runfl.p);
  uint32_t* pos = static_cast<uint32_t*>(ctx->runpos.p);
  gdl::run_flags(ctx->skeys, ctx->sparse, n, fl, ctx->sms, s);
  gdprim::exclusive_scan_u32(fl, pos, n, ctx->scantemp.p, ctx->dM(), s);
  gdl::run_scatter(fl, pos, n, static_cast<int*>(ctx->reps.p), ctx->dM(), ctx->dCtr(), ctx->sms, s);
  if (ctx->sparse) {
    GD_CUDA(cudaMemsetAsync(ctx->hkeys.p, 0xff, hcap * 8, s), "clear cell hash");
    gdl::hash_insert(static_cast<const unsigned long long*>(ctx->skeys),
                     static_cast<int*>(ctx->reps.p), ctx->dM(), n,
                     static_cast<unsigned long long*>(ctx->hkeys.p),
                     static_cast<uint32_t*>(ctx->hvals.p), ctx->hmask, ctx->sms, s);
  } else {
    GD_CUDA(cudaMemsetAsync(ctx->table.p, 0, (C + 1) * 4, s), "clear cell table");
    gdl::cell_counts(static_cast<const uint32_t*>(ctx->skeys), static_cast<int*>(ctx->reps.p),
                     ctx->dM(), n, static_cast<uint32_t*>(ctx->table.p), ctx->sms, s);
    gdprim::exclusive_scan_u32(static_cast<uint32_t*>(ctx->table.p),
                               static_cast<uint32_t*>(ctx->table.p), (int64_t)C + 1,
                               ctx->scantemp.p, nullptr, s);
  }
  cudaEventRecord(ctx->ev[2], s);
  GD_CUDA(cudaGetLastError(), "index build launch");
  {
    const int passes = (ctx->hp.key_bits + 7) / 8;
    // bbox, params, keys, sort, gather, run flags, scan, run scatter, counts, scan
    // bbox, params, keys, sort, gather, run flags, scan, run scatter, table or hash
    ctx->launches = 3 + (passes ? passes * 5 : 1) + 1 + 1 + 3 + 1 + (ctx->sparse ? 1 : 4);
  }
  ctx->st.grid_cells = (int64_t)C;
  ctx->st.key_bits = ctx->hp.key_bits;
  ctx->stage = 1;
  return GD_OK;
}

gd_status gd_expand(gd_ctx* ctx, int32_t minpts) {
  if (!ctx) return fail(GD_EINVAL, "gd_expand: NULL context");
  if (ctx->stage < 1) return fail(GD_ESTATE, "gd_expand: call gd_index_build first");
  if (minpts < 1) return fail(GD_EINVAL, "gd_expand: minpts must be >= 1");
  GD_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t s = ctx->stream;
  const int64_t n = ctx->n;
  ctx->minpts = minpts;
  if (n == 0) {
    ctx->stage = 2;
    return GD_OK;
  }
  gd_status st;
  if ((st = ctx->ensure(ctx->core, n, "core flags")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->cellcore, n * 4, "cell core counts")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->cellmin, n * 4, "cell min index")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->parent, n * 4, "union-find parents")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->Fmark, n * 4, "cluster marks")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->cellcid, n * 4, "cell cluster ids")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->lab, n * 4, "labels")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->asym, gd::kAsymCap * 8, "one-directional links")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->hvcell, n * 4, "heavy-work list")) != GD_OK) return st;
  if ((st = ctx->ensure(ctx->hvmask, n * 8, "heavy-work masks")) != GD_OK) return st;
  size_t sc = gdprim::scan_temp_bytes(n);
  if ((st = ctx->ensure(ctx->scantemp, std::max(sc, ctx->scantemp.bytes), "scan temp")) != GD_OK)
    return st;
  // minpts into the device parameters; counters except the cell count
  ctx->hp.minpts = minpts;
  GD_CUDA(cudaMemcpyAsync(ctx->dP(), &ctx->hp, sizeof(gd::DevParams), cudaMemcpyHostToDevice, s),
          "write parameters");
  GD_CUDA(cudaMemsetAsync(ctx->dCtr() + 1, 0, (gd::kCtrCount - 1) * 8, s), "clear counters");
  gdl::Bufs B = ctx->bufs();
  const int D = ctx->dim;
  cudaEventRecord(ctx->ev[3], s);
  gdl::core(B, n, D, ctx->f32, ctx->sparse, ctx->sms, s);
  cudaEventRecord(ctx->ev[4], s);
  gdl::unite(B, n, D, ctx->f32, ctx->sparse, ctx->sms, s);
  cudaEventRecord(ctx->ev[5], s);
  GD_CUDA(cudaMemsetAsync(B.Fmark, 0, n * 4, s), "clear marks");
  gdl::roots(B, n, ctx->sms, s);
  gdprim::exclusive_scan_u32(B.Fmark, B.Fmark, n, ctx->scantemp.p, ctx->dK(), s);
  gdl::label(B, n, ctx->sms, s);
  gdl::border(B, n, D, ctx->f32, ctx->sparse, ctx->sms, s);
  GD_CUDA(cudaGetLastError(), "expand launch");
  // core (scan+heavy), parent init, 2 union passes (scan+heavy), compress, merge replay,
  // roots, scan, label, border (scan+heavy)
  ctx->launches += 2 + 1 + 4 + 1 + 1 + 1 + 3 + 1 + 2;
  ctx->stage = 2;
  return GD_OK;
}

gd_status gd_get_result(gd_ctx* ctx, int32_t* labels, uint8_t* is_core, int32_t on_device,
                        int64_t* cluster_count, int64_t* noise_count) {
  if (!ctx) return fail(GD_EINVAL, "gd_get_result: NULL context");
  if (ctx->stage < 2) return fail(GD_ESTATE, "gd_get_result: call gd_expand first");
  GD_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t s = ctx->stream;
  const int64_t n = ctx->n;
  gd_stats& S = ctx->st;
  if (n == 0) {
    if (cluster_count) *cluster_count = 0;
    if (noise_count) *noise_count = 0;
    return GD_OK;
  }
  if (!labels) return fail(GD_EINVAL, "gd_get_result: labels is NULL");
  gd_status st;
  int* out = reinterpret_cast<int*>(labels);
  uint8_t* cout = is_core;
  if (!on_device) {
    if ((st = ctx->ensure(ctx->out, n * 4, "label output")) != GD_OK) return st;
    out = static_cast<int*>(ctx->out.p);
    if (is_core) {
      if ((st = ctx->ensure(ctx->coreout, n, "core output")) != GD_OK) return st;
      cout = static_cast<uint8_t*>(ctx->coreout.p);
    }
  }
  GD_CUDA(cudaMemsetAsync(ctx->dCtr() + gd::kCtrCore, 0, 2 * 8, s), "clear counters");
  gdl::Bufs B = ctx->bufs();
  gdl::scatter_labels(B, n, out, cout, ctx->sms, s);
  ++ctx->launches;
  cudaEventRecord(ctx->ev[6], s);
  if (!on_device) {
    GD_CUDA(cudaMemcpyAsync(labels, out, n * 4, cudaMemcpyDeviceToHost, s), "copy labels");
    if (is_core)
      GD_CUDA(cudaMemcpyAsync(is_core, cout, n, cudaMemcpyDeviceToHost, s), "copy core flags");
  }
  cudaEventRecord(ctx->ev[7], s);
  unsigned long long ctr[gd::kCtrCount];
  uint32_t K = 0;
  GD_CUDA(cudaMemcpyAsync(ctr, ctx->dCtr(), sizeof ctr, cudaMemcpyDeviceToHost, s), "counters");
  GD_CUDA(cudaMemcpyAsync(&K, ctx->dK(), 4, cudaMemcpyDeviceToHost, s), "cluster count");
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "DBSCAN pipeline");
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
  if (ctr[gd::kCtrAsymEdges] > (unsigned long long)gd::kAsymCap) {
    ctx->stage = 1;
    return fail(GD_ERANGE, "more one-directional core neighbour pairs than the merge replay "
                           "holds (2048)");
  }
  S.precision_used = ctx->f32 ? GD_PREC_FP32_BAND : GD_PREC_FP64;
  S.launches = ctx->launches;
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
  if (cluster_count) *cluster_count = S.n_clusters;
  if (noise_count) *noise_count = S.n_noise;
  return GD_OK;
}

gd_status gd_dbscan(gd_ctx* ctx, const gd_points* pts, double eps, int32_t minpts,
                    int32_t* labels, gd_stats* stats) {
  if (!ctx || !pts) return fail(GD_EINVAL, "gd_dbscan: NULL argument");
  if (minpts < 1) return fail(GD_EINVAL, "gd_dbscan: minpts must be >= 1");
  gd_status s = gd_index_build(ctx, pts, eps);
  if (s != GD_OK) return s;
  if ((s = gd_expand(ctx, minpts)) != GD_OK) return s;
  if ((s = gd_get_result(ctx, labels, nullptr, pts->on_device, nullptr, nullptr)) != GD_OK)
    return s;
  if (stats) *stats = ctx->st;
  return GD_OK;
}

gd_status gd_get_stats(gd_ctx* ctx, gd_stats* stats) {
  if (!ctx || !stats) return fail(GD_EINVAL, "gd_get_stats: NULL argument");
  *stats = ctx->st;
  return GD_OK;
}

}  // extern "C"
