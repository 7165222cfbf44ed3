// gd_prims.cu -- device primitives: exclusive scan and a stable LSD radix sort.
//
// The scan is a single-pass design with decoupled look-back: each tile
// publishes its aggregate, reads its predecessors' published values back to the
// nearest inclusive prefix, and publishes its own inclusive prefix.  Tiles take
// their index from an atomic counter when their block starts, so a tile only
// waits on tiles that running blocks hold and every wait ends; each wait is
// still bounded (kWaitPolls polls), and a wait that gives up counts the
// predecessor as 0 -- every offset then stays at or below its true value, so no
// write leaves its array -- and is reported through the caller's counter.
//
// Scan (u32): tiles of 8192 elements (512 threads x 16 contiguous items), one
// launch (k_scan_onepass): reads 4 B, writes 4 B/elem.  Against the earlier
// reduce / partials / down-sweep kernels it saves two launches per scan (C2:
// union and label phases about 10 us faster each).
// Radix sort (u32 or u64 key, u32 value), 8- or 9-bit digits, tiles of 4096 pairs
// (256 threads x 16 items; each warp owns a contiguous 512-element segment so
// warp-local ranking in item order is stable):
//   k_rs_upsweep     per-tile digit histograms       reads 4 B/pair
//   exclusive scan over the [digit][tile] histogram (k_scan_onepass)
//   k_rs_downsweep   rank in tile, regroup in shared memory, scatter
//                                                    reads 8 B, writes 8 B/pair
// A onesweep variant (one histogram kernel for all passes, per-digit look-back
// in the scatter kernel) was measured slower on C2 (index phase 0.78 -> 0.94
// ms): with about 760 tiles in flight the serial per-digit look-back chains
// cost more than the upsweep and the histogram scan they replace.
// This replaces thrust::sort_by_key (main.cu:332).
//
// The scan's state between launches lives in the caller's temp memory, which
// must be zero when first used (the callers clear it when they allocate it): a
// control block (tile counter, finished-block counter, launch epoch) that the
// last block of each launch resets, and the status words, tagged with the
// launch's epoch so that words left by earlier launches read as not ready.
#include "gd_internal.cuh"

namespace gdprim {

namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(gd::kFull, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// exclusive scan of one value per thread across a block of NT threads
template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* s_warp,
                                                    uint32_t* block_total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  constexpr int NW = NT / 32;
  uint32_t inc = warp_incl_scan(v, lane);
  if (lane == 31) s_warp[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < NW ? s_warp[lane] : 0u;
    uint32_t ti = warp_incl_scan(t, lane);
    if (lane < NW) s_warp[lane] = ti - t;
    if (lane == NW - 1 && block_total) *block_total = ti;
  }
  __syncthreads();
  uint32_t r = s_warp[w] + inc - v;
  __syncthreads();
  return r;
}

// value of one scanned element: the element itself, or (POPC) the number of
// set bits of a 32-bit word
template <bool POPC>
__device__ __forceinline__ uint32_t scan_val(uint32_t x) {
  return POPC ? (uint32_t)__popc(x) : x;
}

// ------------------------------------------------------------ look-back state
struct LookbackCtl {
  unsigned int tile;   // next tile index of the running launch
  unsigned int done;   // blocks of the running launch that finished
  unsigned int epoch;  // launches completed on this control block
  unsigned int pad[13];
};
static_assert(sizeof(LookbackCtl) == 64, "control block is 64 bytes");

// A predecessor tile's block is already running when its tile is waited on, so
// its aggregate follows within microseconds; 2^14 polls (about 16 ms) only end
// waits that could never succeed.
constexpr unsigned kWaitPolls = 1u << 14;

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// status word: tag (bits 63..34), kind (33..32: 1 aggregate, 2 inclusive
// prefix), value (31..0)
__device__ __forceinline__ unsigned long long lb_word(uint32_t tag, uint32_t kind, uint32_t v) {
  return ((unsigned long long)tag << 34) | ((unsigned long long)kind << 32) | v;
}

// A tile's status word once it carries this launch's tag: its kind (1 or 2)
// and value; kind 0 (value 0) when kWaitPolls polls saw nothing.
__device__ __forceinline__ uint32_t lb_wait(const unsigned long long* p, uint32_t tag,
                                            uint32_t& v) {
  for (unsigned it = 0; it < kWaitPolls; ++it) {
    const unsigned long long w = ld_relaxed_u64(p);
    const uint32_t kind = (uint32_t)(w >> 32) & 3u;
    if ((uint32_t)(w >> 34) == tag && kind != 0u) {
      v = (uint32_t)w;
      return kind;
    }
    if (it >= 4) __nanosleep(64);
  }
  v = 0;
  return 0;
}

// Block start: the tile index (from the counter) and the launch's tag.
__device__ __forceinline__ void lb_begin(LookbackCtl* ctl, unsigned* s_tile, unsigned* s_epoch) {
  if (threadIdx.x == 0) {
    *s_tile = atomicAdd(&ctl->tile, 1u);
    *s_epoch = *reinterpret_cast<volatile unsigned*>(&ctl->epoch);
  }
  __syncthreads();
}

__device__ __forceinline__ uint32_t lb_tag(unsigned epoch) { return (epoch & 0x3fffffffu) + 1u; }

// Block end, after every thread is done with the status words: the last block
// of the launch resets the counters and advances the epoch for the next one.
__device__ __forceinline__ void lb_end(LookbackCtl* ctl, unsigned tiles, unsigned epoch) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ctl->done, 1u) == tiles - 1u) {
      ctl->tile = 0u;
      ctl->done = 0u;
      ctl->epoch = epoch + 1u;
    }
  }
}

// Exclusive prefix of tile `tile` from its predecessors' status words, by one
// warp (32 predecessors per round, nearest first).  *gave_up: a wait ran out.
__device__ __forceinline__ uint32_t lb_warp_prefix(const unsigned long long* status, int64_t tile,
                                                   uint32_t tag, bool* gave_up) {
  const int lane = threadIdx.x & 31;
  uint32_t excl = 0;
  bool lost = false;
  for (int64_t top = tile - 1; top >= 0; top -= 32) {
    const int64_t k = top - lane;
    uint32_t v = 0, kind = 2;  // before tile 0: an inclusive prefix of 0
    if (k >= 0) kind = lb_wait(status + k, tag, v);
    lost |= __any_sync(gd::kFull, kind == 0u);
    // nearest lane holding a prefix (or a wait that gave up): sum up to it
    const unsigned stop = __ballot_sync(gd::kFull, kind != 1u);
    const int last = stop ? __ffs(stop) - 1 : 31;
    uint32_t add = lane <= last ? v : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) add += __shfl_xor_sync(gd::kFull, add, o);
    excl += add;
    if (stop) break;
  }
  *gave_up = lost;
  return excl;
}

// Single-pass exclusive scan (decoupled look-back).
template <bool POPC>
__global__ void __launch_bounds__(kScanThreads)
k_scan_onepass(const uint32_t* in, uint32_t* out, int64_t n, unsigned tiles, LookbackCtl* ctl,
               unsigned long long* status, uint32_t* total_dev, unsigned long long* timeouts) {
  __shared__ uint32_t s_warp[32];
  __shared__ unsigned s_tile, s_epoch;
  __shared__ uint32_t s_agg, s_excl;
  lb_begin(ctl, &s_tile, &s_epoch);
  const unsigned tile = s_tile, epoch = s_epoch;
  const uint32_t tag = lb_tag(epoch);
  if (tile >= tiles) {
    // a counter left inconsistent (never expected): no tile, report it
    if (threadIdx.x == 0 && timeouts) atomicAdd(timeouts, 1ull);
    lb_end(ctl, tiles, epoch);
    return;
  }
  const int64_t base = (int64_t)tile * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  const bool full = base + kScanItems <= n;
  if (full) {
    const uint4* p = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q) {
      const uint4 a = p[q];
      v[4 * q] = a.x; v[4 * q + 1] = a.y; v[4 * q + 2] = a.z; v[4 * q + 3] = a.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) v[i] = base + i < n ? in[base + i] : 0u;
  }
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) v[i] = scan_val<POPC>(v[i]);
  uint32_t sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) sum += v[i];
  uint32_t ex = block_excl_scan<kScanThreads>(sum, s_warp, &s_agg);
  if (threadIdx.x < 32) {
    const uint32_t agg = s_agg;
    unsigned long long* my = status + tile;
    if (threadIdx.x == 0) st_relaxed_u64(my, lb_word(tag, tile == 0 ? 2u : 1u, agg));
    bool lost = false;
    const uint32_t excl = tile == 0 ? 0u : lb_warp_prefix(status, (int64_t)tile, tag, &lost);
    if (threadIdx.x == 0) {
      if (tile != 0) st_relaxed_u64(my, lb_word(tag, 2u, excl + agg));
      s_excl = excl;
      if (lost && timeouts) atomicAdd(timeouts, 1ull);
      if (tile == tiles - 1u && total_dev) *total_dev = excl + agg;
    }
  }
  __syncthreads();
  ex += s_excl;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    uint32_t t = v[i];
    v[i] = ex;
    ex += t;
  }
  if (full) {
    uint4* p = reinterpret_cast<uint4*>(out + base);
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q)
      p[q] = make_uint4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  } else {
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
      if (base + i < n) out[base + i] = v[i];
  }
  lb_end(ctl, tiles, epoch);
}

// ---------------------------------------------------------------- radix sort
constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsMaxBins = 512;  // digits of 8 or 9 bits
// items per thread: 16 for 32-bit keys (4096-pair tiles), 8 for 64-bit keys
template <class K>
constexpr int rs_items() { return sizeof(K) == 4 ? 16 : 8; }
constexpr int kRsMinTile = kRsThreads * 8;

template <class K, int ITEMS, int RB>
__global__ void __launch_bounds__(kRsThreads)
k_rs_upsweep(const K* __restrict__ keys, int64_t n, int shift, uint32_t* __restrict__ hist,
             int64_t T) {
  constexpr int SEG = 32 * ITEMS, TILE = kRsThreads * ITEMS, BINS = 1 << RB;
  constexpr uint32_t MASK = BINS - 1;
  // warp-private digit counts (shared-memory atomics), summed at the end
  __shared__ uint32_t h[kRsWarps][BINS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int ww = 0; ww < kRsWarps; ++ww)
    for (int d = threadIdx.x; d < BINS; d += kRsThreads) h[ww][d] = 0;
  __syncthreads();
  const int64_t seg = (int64_t)blockIdx.x * TILE + w * SEG;
  // every item's key in flight at once, then the counts
  uint32_t d[ITEMS];
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    const int64_t e = seg + i * 32 + lane;
    d[i] = e < n ? (uint32_t)(__ldg(keys + e) >> shift) & MASK : 0xffffffffu;
  }
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
    if (d[i] != 0xffffffffu) atomicAdd(&h[w][d[i]], 1u);
  __syncthreads();
  for (int d = threadIdx.x; d < BINS; d += kRsThreads) {
    uint32_t tot = 0;
#pragma unroll
    for (int ww = 0; ww < kRsWarps; ++ww) tot += h[ww][d];
    hist[(int64_t)d * T + blockIdx.x] = tot;
  }
}

template <class K, int ITEMS, int RB>
__global__ void __launch_bounds__(kRsThreads)
k_rs_downsweep(const K* __restrict__ kin, const uint32_t* __restrict__ vin,
               K* __restrict__ kout, uint32_t* __restrict__ vout, int64_t n,
               int shift, const uint32_t* __restrict__ goff, int64_t T) {
  constexpr int SEG = 32 * ITEMS, TILE = kRsThreads * ITEMS, BINS = 1 << RB;
  constexpr int BPT = BINS / kRsThreads;  // digits per thread in the tile scan
  constexpr uint32_t MASK = BINS - 1;
  static_assert(TILE <= 65535, "per-warp digit offsets are 16-bit");
  __shared__ K s_keys[TILE];
  __shared__ uint32_t s_vals[TILE];
  __shared__ uint16_t s_cnt[kRsWarps][BINS];  // per-warp digit counts, then offsets
  __shared__ uint32_t s_dstart[BINS];
  __shared__ int32_t s_gbase[BINS];
  __shared__ uint32_t s_warp[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * TILE;
  const int valid_count = (int)min((int64_t)TILE, n - base);
  for (int i = lane; i < BINS; i += 32) s_cnt[w][i] = 0;
  __syncwarp();
  const unsigned lt_mask = (1u << lane) - 1u;
  K k[ITEMS];
  uint32_t v[ITEMS], r[ITEMS];
  const int64_t seg = base + w * SEG;
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    int64_t e = seg + i * 32 + lane;
    if (e < n) {
      k[i] = __ldg(kin + e);
      v[i] = vin ? __ldg(vin + e) : (uint32_t)e;
    } else {
      k[i] = ~(K)0;
      v[i] = 0;
    }
  }
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    uint32_t d = (uint32_t)(k[i] >> shift) & MASK;
    // lanes holding the same digit: one ballot per digit bit (measured faster
    // than __match_any_sync here)
    unsigned peers = gd::kFull;
#pragma unroll
    for (int bit = 0; bit < RB; ++bit) {
      const unsigned bb = __ballot_sync(gd::kFull, (d >> bit) & 1u);
      peers &= ((d >> bit) & 1u) ? bb : ~bb;
    }
    uint32_t b = s_cnt[w][d];
    __syncwarp();
    if (lane == __ffs(peers) - 1) s_cnt[w][d] = (uint16_t)(b + (uint32_t)__popc(peers));
    __syncwarp();
    r[i] = b + (uint32_t)__popc(peers & lt_mask);
  }
  __syncthreads();
  {
    // digits threadIdx.x * BPT .. + BPT - 1: offsets across warps, then the
    // tile's digit starts
    uint32_t tots[BPT], sum = 0;
#pragma unroll
    for (int q = 0; q < BPT; ++q) {
      const int d = threadIdx.x * BPT + q;
      uint32_t tot = 0;
#pragma unroll
      for (int ww = 0; ww < kRsWarps; ++ww) {
        const uint32_t c = s_cnt[ww][d];
        s_cnt[ww][d] = (uint16_t)tot;
        tot += c;
      }
      tots[q] = tot;
      sum += tot;
    }
    uint32_t ex = block_excl_scan<kRsThreads>(sum, s_warp, nullptr);
#pragma unroll
    for (int q = 0; q < BPT; ++q) {
      const int d = threadIdx.x * BPT + q;
      s_dstart[d] = ex;
      s_gbase[d] = (int32_t)goff[(int64_t)d * T + blockIdx.x] - (int32_t)ex;
      ex += tots[q];
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    uint32_t d = (uint32_t)(k[i] >> shift) & MASK;
    uint32_t pos = s_dstart[d] + s_cnt[w][d] + r[i];
    s_keys[pos] = k[i];
    s_vals[pos] = v[i];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < valid_count; j += kRsThreads) {
    K key = s_keys[j];
    uint32_t d = (uint32_t)(key >> shift) & MASK;
    int64_t g = (int64_t)s_gbase[d] + j;
    kout[g] = key;
    vout[g] = s_vals[j];
  }
}

// positions of the set bits, in order: out[pre[w] + r] = 32 w + (bit r of word
// w).  A warp takes 32 words (one per lane), then writes them one word at a
// time with a lane per bit, so each word's entries go out in one store.
__global__ void k_compact_bits(const uint32_t* __restrict__ words,
                               const uint32_t* __restrict__ pre, int64_t nw,
                               uint32_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;  // 32 words per warp
  for (int64_t w0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); w0 < nw;
       w0 += step) {
    const int64_t w = w0 + lane;
    const uint32_t x = w < nw ? words[w] : 0u;
    const uint32_t p = w < nw ? pre[w] : 0u;
    unsigned busy = __ballot_sync(gd::kFull, x != 0u);
    while (busy) {
      const int src = __ffs(busy) - 1;
      busy &= busy - 1;
      const uint32_t xs = __shfl_sync(gd::kFull, x, src);
      const uint32_t ps = __shfl_sync(gd::kFull, p, src);
      if ((xs >> lane) & 1u)
        out[ps + (uint32_t)__popc(xs & below)] = (uint32_t)((w0 + src) << 5) + (uint32_t)lane;
    }
  }
}

__global__ void k_iota(uint32_t* v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (uint32_t)i;
}

inline size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// temp layout of both primitives: control block (64 B), then their arrays
size_t scan_temp_bytes(int64_t n) {
  const int64_t T = (n + kScanTile - 1) / kScanTile;
  return align_up(sizeof(LookbackCtl) + (size_t)(T > 0 ? T : 1) * 8);
}

int scan_launches(int64_t n) { return n > 0 ? 1 : 0; }

template <bool POPC>
void scan_impl(const uint32_t* in, uint32_t* out, int64_t n, void* temp, uint32_t* total_dev,
               cudaStream_t s, unsigned long long* timeouts) {
  if (n <= 0) {
    if (total_dev) cudaMemsetAsync(total_dev, 0, sizeof(uint32_t), s);
    return;
  }
  const int64_t T = (n + kScanTile - 1) / kScanTile;
  LookbackCtl* ctl = static_cast<LookbackCtl*>(temp);
  unsigned long long* status =
      reinterpret_cast<unsigned long long*>(static_cast<char*>(temp) + sizeof(LookbackCtl));
  k_scan_onepass<POPC><<<(unsigned)T, kScanThreads, 0, s>>>(in, out, n, (unsigned)T, ctl, status,
                                                            total_dev, timeouts);
}

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, void* temp,
                        uint32_t* total_dev, cudaStream_t s, unsigned long long* timeouts) {
  scan_impl<false>(in, out, n, temp, total_dev, s, timeouts);
}

void exclusive_scan_popc(const uint32_t* words, uint32_t* pre, int64_t nw, void* temp,
                         uint32_t* total_dev, cudaStream_t s, unsigned long long* timeouts) {
  scan_impl<true>(words, pre, nw, temp, total_dev, s, timeouts);
}

void compact_bits(const uint32_t* words, const uint32_t* pre, int64_t nw, uint32_t* out, int sms,
                  cudaStream_t s) {
  if (nw <= 0) return;
  int64_t g = (nw + 255) / 256;
  if (g > (int64_t)sms * 8) g = (int64_t)sms * 8;
  k_compact_bits<<<(unsigned)g, 256, 0, s>>>(words, pre, nw, out);
}

// sort temp: the histogram scan's state (its control block at offset 0 for
// every sort on this temp), then the [digit][tile] histogram
size_t sort_temp_bytes(int64_t n) {
  const int64_t T = (n + kRsMinTile - 1) / kRsMinTile;
  const int64_t h = T * kRsMaxBins;
  return scan_temp_bytes(h) + align_up((size_t)h * sizeof(uint32_t));
}

template <class K, int RB>
int sort_passes(K* keys[2], uint32_t* vals[2], int64_t n, int passes, bool vals_in_is_iota,
                void* temp, cudaStream_t s, unsigned long long* timeouts) {
  constexpr int ITEMS = rs_items<K>();
  constexpr int TILE = kRsThreads * ITEMS;
  const int64_t T = (n + TILE - 1) / TILE;
  const int64_t h = T << RB;
  void* scan_temp = temp;
  uint32_t* hist = reinterpret_cast<uint32_t*>(static_cast<char*>(temp) + scan_temp_bytes(h));
  int cur = 0;
  for (int p = 0; p < passes; ++p) {
    int shift = RB * p;
    k_rs_upsweep<K, ITEMS, RB><<<(unsigned)T, kRsThreads, 0, s>>>(keys[cur], n, shift, hist, T);
    exclusive_scan_u32(hist, hist, h, scan_temp, nullptr, s, timeouts);
    const uint32_t* vin = (p == 0 && vals_in_is_iota) ? nullptr : vals[cur];
    k_rs_downsweep<K, ITEMS, RB><<<(unsigned)T, kRsThreads, 0, s>>>(
        keys[cur], vin, keys[cur ^ 1], vals[cur ^ 1], n, shift, hist, T);
    cur ^= 1;
  }
  return cur;
}

int sort_digit_bits(int bits) { return (bits + 8) / 9 < (bits + 7) / 8 ? 9 : 8; }

int sort_launches(int64_t n, int bits) {
  if (n <= 0) return 0;
  const int rb = sort_digit_bits(bits);
  const int passes = (bits + rb - 1) / rb;
  return passes ? passes * 3 : 1;  // upsweep, scan, downsweep per pass
}

// Digits of 9 bits where they save a pass (a 26-bit key: 3 passes, not 4),
// else of 8 bits.
template <class K>
int radix_sort_pairs(K* keys[2], uint32_t* vals[2], int64_t n, int bits, bool vals_in_is_iota,
                     void* temp, cudaStream_t s, unsigned long long* timeouts) {
  if (n <= 0) return 0;
  const int rb = sort_digit_bits(bits);
  const int passes = (bits + rb - 1) / rb;
  if (passes == 0) {
    if (vals_in_is_iota) k_iota<<<1024, 256, 0, s>>>(vals[0], n);
    return 0;
  }
  return rb == 9 ? sort_passes<K, 9>(keys, vals, n, passes, vals_in_is_iota, temp, s, timeouts)
                 : sort_passes<K, 8>(keys, vals, n, passes, vals_in_is_iota, temp, s, timeouts);
}

template int radix_sort_pairs<uint32_t>(uint32_t* [2], uint32_t* [2], int64_t, int, bool, void*,
                                        cudaStream_t, unsigned long long*);
template int radix_sort_pairs<unsigned long long>(unsigned long long* [2], uint32_t* [2], int64_t,
                                                  int, bool, void*, cudaStream_t,
                                                  unsigned long long*);

}  // namespace gdprim
