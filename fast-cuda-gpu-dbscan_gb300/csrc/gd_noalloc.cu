// gd_noalloc.cu -- gd_dbscan_noalloc: exact DBSCAN for small point sets that
// allocates no memory at all.
//
// Who needs it: callers that cannot call cudaMalloc/cudaFree.  Control and
// real-time loops reserve all their device memory at start-up, because an
// allocation can block for milliseconds and cudaFree waits for the whole
// device; plug-ins that run inside a host process whose memory manager owns
// the GPU's memory may not allocate behind its back.  They pass device
// pointers for the points and the labels; every other buffer of the pipeline
// lives in one file-scope __device__ array (kScratchBytes, about 5 MiB) that
// the module holds on every GPU that loads this library until the process
// exits.
//
// Limits and rules:
//   * n <= GD_NOALLOC_MAX_POINTS (32768); larger inputs are rejected with
//     GD_ERANGE.  Grids of more than 8*32768 cells use the hash of occupied
//     cells instead of the dense table, so any extent fits.
//   * The first call in a CUDA context of a device looks the array's device
//     address up (cudaGetSymbolAddress, with that device current) and caches it
//     with the context's id; a new context on that device (after
//     cudaDeviceReset, say) repeats the look-up.  Make that first call before
//     any stream capture begins.
//   * All calls share the one array and it keeps the previous call's contents:
//     everything that must start at zero (counters, flags, cluster marks, the
//     cell table or hash) is cleared inside each call.  Calls whose work
//     overlaps on the GPU (two host threads, or two streams) race on the array
//     and must be serialised by the caller.
//   * The call synchronises its stream twice: once in the middle, to read the
//     grid layout back to the host, and once at the end.  It uses the same
//     kernels as gd_dbscan, so the labels are identical.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda.h>

#include "gbdbscan.h"
#include "gd_launch.h"

namespace gdio {
void set_error(const std::string& m);
}

namespace {

constexpr int64_t kMaxPoints = GD_NOALLOC_MAX_POINTS;
constexpr uint64_t kTableCells = 8ull * kMaxPoints;      // dense table limit
constexpr uint64_t kHashSlots = 2ull * kMaxPoints;       // power of two

constexpr size_t up(size_t x) { return (x + 255) & ~(size_t)255; }

// byte offsets of the buffers inside the scratch array
constexpr int kMaxChunks = (int)((kMaxPoints + gd::kChunkPoints - 1) / gd::kChunkPoints);
constexpr size_t kOffSmall = 0;                                   // M | K | counters
constexpr size_t kOffInst = kOffSmall + 4096;
constexpr size_t kOffChunks = kOffInst + up(sizeof(gd::InstDesc));
constexpr size_t kOffPv = kOffChunks + up(kMaxChunks * sizeof(gd::Chunk));
constexpr size_t kOffBi = kOffPv + up(sizeof(gd::DevParams));
constexpr size_t kOffBbox = kOffBi + up(sizeof(gd::BatchInfo));
constexpr size_t kOffKeys0 = kOffBbox + up(6 * 8);
constexpr size_t kOffKeys1 = kOffKeys0 + up(kMaxPoints * 8);
constexpr size_t kOffVals0 = kOffKeys1 + up(kMaxPoints * 8);
constexpr size_t kOffVals1 = kOffVals0 + up(kMaxPoints * 4);
constexpr size_t kOffX = kOffVals1 + up(kMaxPoints * 4);
constexpr size_t kOffXf = kOffX + up(kMaxPoints * 3 * 8);
constexpr size_t kOffTable = kOffXf + up(kMaxPoints * 3 * 4);
constexpr size_t kOffOcc = kOffTable + up((kTableCells + 1) * 4);
// occupancy, core occupancy, word prefix counts
constexpr size_t kOffHkeys = kOffOcc + up((3 * (kTableCells / 32 + 1) + 64) * 4);
constexpr size_t kOffHvals = kOffHkeys + up(kHashSlots * 8);
constexpr size_t kOffReps = kOffHvals + up(kHashSlots * 8);
constexpr size_t kOffCellz = kOffReps + up((kMaxPoints + 1) * 4);
constexpr size_t kOffBits = kOffCellz + up(kMaxPoints * 4);    // cell starts, lists, marks
constexpr size_t kOffCore = kOffBits + up(gdl::bit_layout(kMaxPoints).words * 4);
constexpr size_t kOffCellcore = kOffCore + up(kMaxPoints);
constexpr size_t kOffCellmin = kOffCellcore + up(kMaxPoints * 4);
constexpr size_t kOffParent = kOffCellmin + up(kMaxPoints * 4);
constexpr size_t kOffCellcid = kOffParent + up(kMaxPoints * 4);
constexpr size_t kOffLab = kOffCellcid + up(kMaxPoints * 4);
constexpr size_t kOffAsym = kOffLab + up(kMaxPoints * 4);
constexpr size_t kOffHvCell = kOffAsym + up(gd::kAsymCap * 8);
constexpr size_t kOffHvMask = kOffHvCell + up(kMaxPoints * 4);
constexpr size_t kOffSortTemp = kOffHvMask + up(kMaxPoints * 8);
constexpr size_t kSortTempBytes = 64 * 1024;   // >= sort_temp_bytes(kMaxPoints), checked below
constexpr size_t kOffScanTemp = kOffSortTemp + kSortTempBytes;
constexpr size_t kScanTempBytes = 4096;        // >= scan_temp_bytes(kTableCells + 1), checked below
constexpr size_t kScratchBytes = kOffScanTemp + kScanTempBytes;

// The scratch.  In host code this name is only a stand-in for the symbol, not
// a device address: kernels get the address from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
// per device: the scratch address and the id of the CUDA context it belongs to
unsigned char* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

// Driver functions that identify the current context, reached through the
// runtime (the library does not link the driver library itself).
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

gd_status fail(gd_status s, const std::string& m) {
  gdio::set_error(m);
  return s;
}

gd_status cuda_fail(cudaError_t e, const char* what) {
  return fail(GD_ECUDA, std::string("gd_dbscan_noalloc: ") + what + ": " + cudaGetErrorString(e));
}

#define NA_CUDA(call, what)                            \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

// Id of the CUDA context current on the calling thread (0 when none is).
gd_status current_ctx_id(unsigned long long* id) {
  *id = 0;
  if (!g_ctx_get_current || !g_ctx_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) !=
            cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) !=
            cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
      cudaGetLastError();
      return fail(GD_ECUDA, "gd_dbscan_noalloc: driver context functions unavailable");
    }
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext c = nullptr;
  if (g_ctx_get_current(&c) != CUDA_SUCCESS)
    return fail(GD_ECUDA, "gd_dbscan_noalloc: cuCtxGetCurrent failed");
  if (c && g_ctx_get_id(c, id) != CUDA_SUCCESS)
    return fail(GD_ECUDA, "gd_dbscan_noalloc: cuCtxGetId failed");
  return GD_OK;
}

// Device address of the scratch array on the current device.  Set up once per
// CUDA context of a device, with that device current: the address is looked up
// and cached with the context's id, and looked up again only when another
// context has become current on the device (the module, and with it the array,
// is loaded anew in every context).
gd_status scratch_of(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  unsigned long long id = 0;
  gd_status st = current_ctx_id(&id);
  if (st != GD_OK) return st;
  if (!g_scratch_ptr[dev] || id == 0 || id != g_scratch_ctx[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
    // the look-up made the device's primary context current if none was
    st = current_ctx_id(&id);
    if (st != GD_OK) return st;
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    g_scratch_ctx[dev] = id;
  }
  *out = g_scratch_ptr[dev];
  return GD_OK;
}

}  // namespace

extern "C" gd_status gd_dbscan_noalloc(const double* coords_dev, int64_t n, int32_t dim,
                                       double eps, int32_t minpts, int32_t precision,
                                       int32_t* labels_dev, int64_t* n_clusters, void* stream) {
  if (n < 0 || (dim != 2 && dim != 3))
    return fail(GD_EINVAL, "gd_dbscan_noalloc: n must be >= 0 and dim 2 or 3");
  if (n > kMaxPoints)
    return fail(GD_ERANGE, "gd_dbscan_noalloc: n = " + std::to_string(n) +
                               " exceeds the fixed scratch capacity of " +
                               std::to_string(kMaxPoints) + " points; use gd_dbscan");
  if (!(eps > 0) || eps != eps || eps > 1.7e308)
    return fail(GD_EINVAL, "gd_dbscan_noalloc: eps must be positive and finite");
  if (minpts < 1) return fail(GD_EINVAL, "gd_dbscan_noalloc: minpts must be >= 1");
  if (precision != GD_PREC_FP64 && precision != GD_PREC_FP32_BAND)
    return fail(GD_EINVAL, "gd_dbscan_noalloc: unknown precision mode");
  if (n > 0 && (!coords_dev || !labels_dev))
    return fail(GD_EINVAL, "gd_dbscan_noalloc: NULL pointer");
  if (n_clusters) *n_clusters = 0;
  if (n == 0) return GD_OK;
  if (gdprim::sort_temp_bytes(kMaxPoints) > kSortTempBytes ||
      gdprim::scan_temp_bytes((int64_t)kTableCells + 1) > kScanTempBytes ||
      gdprim::scan_temp_bytes(kMaxPoints + 1) > kScanTempBytes)
    return fail(GD_EINVAL, "gd_dbscan_noalloc: scratch layout inconsistent (build error)");

  int dev = 0;
  NA_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(GD_ENODEV, "gd_dbscan_noalloc: device index");
  int sms = 0;
  NA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  unsigned char* base = nullptr;
  gd_status st = scratch_of(dev, &base);
  if (st != GD_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  uint32_t* dM = reinterpret_cast<uint32_t*>(base + kOffSmall);
  uint32_t* dK = reinterpret_cast<uint32_t*>(base + kOffSmall + 4);
  unsigned long long* dCtr = reinterpret_cast<unsigned long long*>(base + kOffSmall + 128);

  // the run description: one instance, chunks of kChunkPoints points
  gd::InstDesc desc{0, n, 0, eps, dim, minpts};
  gd::Chunk chunks[kMaxChunks];
  int nch = 0;
  for (int64_t b = 0; b < n; b += gd::kChunkPoints, ++nch)
    chunks[nch] = gd::Chunk{0, 0, b, std::min<int64_t>(n, b + gd::kChunkPoints)};
  NA_CUDA(cudaMemsetAsync(base + kOffSmall, 0, 4096, s), "clear counters");
  NA_CUDA(cudaMemsetAsync(base + kOffBi, 0, sizeof(gd::BatchInfo), s), "clear layout");
  NA_CUDA(cudaMemcpyAsync(base + kOffInst, &desc, sizeof desc, cudaMemcpyHostToDevice, s),
          "upload instance");
  NA_CUDA(cudaMemcpyAsync(base + kOffChunks, chunks, nch * sizeof(gd::Chunk),
                          cudaMemcpyHostToDevice, s), "upload chunks");
  gdl::Bufs B;
  B.coords = coords_dev;
  B.inst = reinterpret_cast<const gd::InstDesc*>(base + kOffInst);
  B.chunks = reinterpret_cast<const gd::Chunk*>(base + kOffChunks);
  B.Pv = reinterpret_cast<gd::DevParams*>(base + kOffPv);
  B.Bi = reinterpret_cast<gd::BatchInfo*>(base + kOffBi);
  B.bbox = reinterpret_cast<long long*>(base + kOffBbox);
  B.M = dM;
  B.ctr = dCtr;
  // index build (the same stages as gd_index_build)
  gdl::grids(B, 1, nch, 0.5 * (1.0 + 1.0 / 65536.0), 0.5 * (1.0 + 1.0 / 65536.0), kTableCells,
             0, s);
  gd::BatchInfo bi;
  NA_CUDA(cudaMemcpyAsync(&bi, base + kOffBi, sizeof bi, cudaMemcpyDeviceToHost, s),
          "read run layout");
  NA_CUDA(cudaStreamSynchronize(s), "grid parameters");
  if (bi.flags & gd::kFlagNonFinite)
    return fail(GD_EINVAL, "gd_dbscan_noalloc: input has NaN or Inf coordinates");
  if (bi.flags & gd::kFlagGridTooLarge)
    return fail(GD_ERANGE, "gd_dbscan_noalloc: eps-cell grid too large");
  const bool f32 = precision == GD_PREC_FP32_BAND && !bi.band_off;
  const bool key64 = bi.key64 != 0;
  const bool xf = f32 || bi.any_xf;
  const int dims = dim == 2 ? 1 : 2;
  const int key_bits = bi.LB + bi.IB;
  gdl::keys(B, key64, nch, base + kOffKeys0, s);
  uint32_t* vb[2] = {reinterpret_cast<uint32_t*>(base + kOffVals0),
                     reinterpret_cast<uint32_t*>(base + kOffVals1)};
  const void* skeys;
  int r;
  if (key64) {
    using U64 = unsigned long long;
    U64* kb[2] = {reinterpret_cast<U64*>(base + kOffKeys0), reinterpret_cast<U64*>(base + kOffKeys1)};
    r = gdprim::radix_sort_pairs<U64>(kb, vb, n, key_bits, true, base + kOffSortTemp, s,
                                      dCtr + gd::kCtrWaitTimeouts);
    skeys = kb[r];
  } else {
    uint32_t* kb[2] = {reinterpret_cast<uint32_t*>(base + kOffKeys0),
                       reinterpret_cast<uint32_t*>(base + kOffKeys1)};
    r = gdprim::radix_sort_pairs<uint32_t>(kb, vb, n, key_bits, true, base + kOffSortTemp, s,
                                           dCtr + gd::kCtrWaitTimeouts);
    skeys = kb[r];
  }
  B.keys = skeys;
  B.ids = vb[r];
  B.blist = vb[1 - r];  // the sort's other id and key buffers are free after the sort
  gdl::set_bits(B, reinterpret_cast<uint32_t*>(base + kOffBits), n);
  B.K = dK;
  B.X = reinterpret_cast<double*>(base + kOffX);
  B.Xf = reinterpret_cast<float*>(base + kOffXf);
  B.reps = reinterpret_cast<int*>(base + kOffReps);
  B.cellz = reinterpret_cast<uint32_t*>(base + kOffCellz);
  B.start = reinterpret_cast<uint32_t*>(base + kOffTable);
  B.occ = reinterpret_cast<uint32_t*>(base + kOffOcc);
  if (bi.occ_total) {
    B.occ_words = bi.occ_total / 32 + 1;
    B.cocc = B.occ + B.occ_words;
    B.wpre = B.occ + gdl::occ_wpre_offset(B.occ_words);
  }
  B.hkeys = reinterpret_cast<unsigned long long*>(base + kOffHkeys);
  B.hvals = reinterpret_cast<uint32_t*>(base + kOffHvals);
  B.hmask = (uint32_t)(kHashSlots - 1);
  gdl::gather(B, key64, n, xf, true, sms, s);
  gdl::runs(B, key64, n, false, sms, base + kOffScanTemp, s);
  NA_CUDA(cudaMemsetAsync(B.start, 0, bi.start_total * 4, s), "clear row table");
  if (B.occ_words) NA_CUDA(cudaMemsetAsync(B.occ, 0, B.occ_words * 4, s), "clear occupancy");
  gdl::cell_counts(B, key64, n, sms, s);
  gdl::start_fill(B, 1, s);
  gdprim::exclusive_scan_u32(B.start, B.start, (int64_t)bi.start_total, base + kOffScanTemp,
                             nullptr, s, dCtr + gd::kCtrWaitTimeouts);
  gdl::occ_rank(B, 1, base + kOffScanTemp, s);
  if (bi.any_sparse) {
    NA_CUDA(cudaMemsetAsync(B.hkeys, 0xff, kHashSlots * 8, s), "clear row hash");
    gdl::hash_insert(B, key64, n, sms, s);
  }

  // expansion (the same stages as gd_expand)
  B.core = base + kOffCore;
  B.cellcore = reinterpret_cast<int*>(base + kOffCellcore);
  B.cellmin = reinterpret_cast<int*>(base + kOffCellmin);
  B.parent = reinterpret_cast<int*>(base + kOffParent);
  B.cellcid = reinterpret_cast<int*>(base + kOffCellcid);
  B.lab = reinterpret_cast<int*>(base + kOffLab);
  B.asym = reinterpret_cast<int*>(base + kOffAsym);
  B.hv_cell = reinterpret_cast<int*>(base + kOffHvCell);
  B.hv_mask = reinterpret_cast<unsigned long long*>(base + kOffHvMask);
  gdl::core(B, n, dims, f32, key64, true, sms, base + kOffScanTemp, s);
  gdl::unite(B, n, dims, f32, key64, sms, base + kOffScanTemp, s);
  gdl::roots(B, key64, n, sms, base + kOffScanTemp, s);
  gdl::label(B, n, sms, base + kOffScanTemp, s);
  gdl::border(B, n, dims, f32, key64, sms, s);
  gdl::scatter_labels(B, n, labels_dev, nullptr, sms, s);
  NA_CUDA(cudaGetLastError(), "launch");
  unsigned long long ctr[gd::kCtrCount];
  uint32_t K = 0;
  NA_CUDA(cudaMemcpyAsync(ctr, dCtr, sizeof ctr, cudaMemcpyDeviceToHost, s), "read counters");
  NA_CUDA(cudaMemcpyAsync(&K, dK, 4, cudaMemcpyDeviceToHost, s), "read cluster count");
  NA_CUDA(cudaStreamSynchronize(s), "DBSCAN pipeline");
  if (ctr[gd::kCtrWaitTimeouts]) {
    // start the scan and sort state afresh for the next call
    cudaMemsetAsync(base + kOffSortTemp, 0, kSortTempBytes + kScanTempBytes, s);
    cudaStreamSynchronize(s);
    return fail(GD_ECUDA, "gd_dbscan_noalloc: a scan or sort look-back wait gave up");
  }
  if (ctr[gd::kCtrAsymEdges] > (unsigned long long)gd::kAsymCap)
    return fail(GD_ERANGE, "gd_dbscan_noalloc: too many one-directional core neighbour pairs");
  if (n_clusters) *n_clusters = K;
  return GD_OK;
}
