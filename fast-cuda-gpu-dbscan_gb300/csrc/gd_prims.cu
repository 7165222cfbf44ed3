// gd_prims.cu -- device primitives: exclusive scan and a stable LSD radix sort.
//
// Both are reduce-then-scan designs: no kernel waits on another block, so no
// spin loop exists anywhere in them.
//
// Scan (u32): tiles of 4096 elements (512 threads x 8 contiguous items).
//   k_scan_reduce    tile sums                       reads 4 B/elem
//   k_scan_partials  one block scans the tile sums
//   k_scan_down      tile-local scan + tile offset   reads 4 B, writes 4 B/elem
// Radix sort (u32 or u64 key, u32 value), 8- or 9-bit digits, tiles of 4096 pairs
// (256 threads x 16 items; each warp owns a contiguous 512-element segment so
// warp-local ranking in item order is stable):
//   k_rs_upsweep     per-tile digit histograms       reads 4 B/pair
//   exclusive scan over the [digit][tile] histogram
//   k_rs_downsweep   rank in tile, regroup in shared memory, scatter
//                                                    reads 8 B, writes 8 B/pair
// This replaces thrust::sort_by_key (main.cu:332).
#include "gd_internal.cuh"

namespace gdprim {

namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
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

template <bool POPC>
__global__ void __launch_bounds__(kScanThreads)
k_scan_reduce(const uint32_t* __restrict__ in, int64_t n, uint32_t* __restrict__ partial) {
  __shared__ uint32_t s_warp[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t sum = 0;
  if (base + kScanItems <= n) {
    const uint4* p = reinterpret_cast<const uint4*>(in + base);
    uint4 a = p[0], b = p[1];
    sum = scan_val<POPC>(a.x) + scan_val<POPC>(a.y) + scan_val<POPC>(a.z) + scan_val<POPC>(a.w) +
          scan_val<POPC>(b.x) + scan_val<POPC>(b.y) + scan_val<POPC>(b.z) + scan_val<POPC>(b.w);
  } else {
    for (int i = 0; i < kScanItems; ++i)
      if (base + i < n) sum += scan_val<POPC>(in[base + i]);
  }
  // block reduction
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(gd::kFull, sum, o);
  if (lane == 0) s_warp[w] = sum;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < kScanThreads / 32 ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(gd::kFull, t, o);
    if (lane == 0) partial[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(1024)
k_scan_partials(uint32_t* partial, int64_t T, uint32_t* total_dev) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  uint32_t carry = 0;
  for (int64_t base = 0; base < T; base += 1024) {
    int64_t i = base + threadIdx.x;
    uint32_t v = i < T ? partial[i] : 0u;
    uint32_t ex = block_excl_scan<1024>(v, s_warp, &s_total);
    if (i < T) partial[i] = carry + ex;
    __syncthreads();
    carry += s_total;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total_dev) *total_dev = carry;
}

template <bool POPC>
__global__ void __launch_bounds__(kScanThreads)
k_scan_down(const uint32_t* in, uint32_t* out, int64_t n, const uint32_t* __restrict__ partial) {
  __shared__ uint32_t s_warp[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  const bool full = base + kScanItems <= n;
  if (full) {
    const uint4* p = reinterpret_cast<const uint4*>(in + base);
    uint4 a = p[0], b = p[1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else {
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) v[i] = base + i < n ? in[base + i] : 0u;
  }
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) v[i] = scan_val<POPC>(v[i]);
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) s += v[i];
  uint32_t ex = block_excl_scan<kScanThreads>(s, s_warp, nullptr) + partial[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    uint32_t t = v[i];
    v[i] = ex;
    ex += t;
  }
  if (full) {
    uint4* p = reinterpret_cast<uint4*>(out + base);
    p[0] = make_uint4(v[0], v[1], v[2], v[3]);
    p[1] = make_uint4(v[4], v[5], v[6], v[7]);
  } else {
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
      if (base + i < n) out[base + i] = v[i];
  }
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

size_t scan_temp_bytes(int64_t n) {
  int64_t T = (n + kScanTile - 1) / kScanTile;
  return align_up((size_t)(T + 1) * sizeof(uint32_t));
}

template <bool POPC>
void scan_impl(const uint32_t* in, uint32_t* out, int64_t n, void* temp, uint32_t* total_dev,
               cudaStream_t s) {
  if (n <= 0) {
    if (total_dev) cudaMemsetAsync(total_dev, 0, sizeof(uint32_t), s);
    return;
  }
  int64_t T = (n + kScanTile - 1) / kScanTile;
  uint32_t* partial = static_cast<uint32_t*>(temp);
  k_scan_reduce<POPC><<<(unsigned)T, kScanThreads, 0, s>>>(in, n, partial);
  k_scan_partials<<<1, 1024, 0, s>>>(partial, T, total_dev);
  k_scan_down<POPC><<<(unsigned)T, kScanThreads, 0, s>>>(in, out, n, partial);
}

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, void* temp,
                        uint32_t* total_dev, cudaStream_t s) {
  scan_impl<false>(in, out, n, temp, total_dev, s);
}

void exclusive_scan_popc(const uint32_t* words, uint32_t* pre, int64_t nw, void* temp,
                         uint32_t* total_dev, cudaStream_t s) {
  scan_impl<true>(words, pre, nw, temp, total_dev, s);
}

void compact_bits(const uint32_t* words, const uint32_t* pre, int64_t nw, uint32_t* out, int sms,
                  cudaStream_t s) {
  if (nw <= 0) return;
  int64_t g = (nw + 255) / 256;
  if (g > (int64_t)sms * 8) g = (int64_t)sms * 8;
  k_compact_bits<<<(unsigned)g, 256, 0, s>>>(words, pre, nw, out);
}

size_t sort_temp_bytes(int64_t n) {
  int64_t T = (n + kRsMinTile - 1) / kRsMinTile;
  int64_t h = T * kRsMaxBins;
  return align_up((size_t)h * sizeof(uint32_t)) + scan_temp_bytes(h);
}

template <class K, int RB>
int sort_passes(K* keys[2], uint32_t* vals[2], int64_t n, int passes, bool vals_in_is_iota,
                void* temp, cudaStream_t s) {
  constexpr int ITEMS = rs_items<K>();
  constexpr int TILE = kRsThreads * ITEMS;
  int64_t T = (n + TILE - 1) / TILE;
  int64_t h = T << RB;
  uint32_t* hist = static_cast<uint32_t*>(temp);
  void* scan_temp = static_cast<char*>(temp) + align_up((size_t)h * sizeof(uint32_t));
  int cur = 0;
  for (int p = 0; p < passes; ++p) {
    int shift = RB * p;
    k_rs_upsweep<K, ITEMS, RB><<<(unsigned)T, kRsThreads, 0, s>>>(keys[cur], n, shift, hist, T);
    exclusive_scan_u32(hist, hist, h, scan_temp, nullptr, s);
    const uint32_t* vin = (p == 0 && vals_in_is_iota) ? nullptr : vals[cur];
    k_rs_downsweep<K, ITEMS, RB><<<(unsigned)T, kRsThreads, 0, s>>>(
        keys[cur], vin, keys[cur ^ 1], vals[cur ^ 1], n, shift, hist, T);
    cur ^= 1;
  }
  return cur;
}

int sort_digit_bits(int bits) { return (bits + 8) / 9 < (bits + 7) / 8 ? 9 : 8; }

// Digits of 9 bits where they save a pass (a 26-bit key: 3 passes, not 4),
// else of 8 bits.
template <class K>
int radix_sort_pairs(K* keys[2], uint32_t* vals[2], int64_t n, int bits, bool vals_in_is_iota,
                     void* temp, cudaStream_t s) {
  if (n <= 0) return 0;
  const int rb = sort_digit_bits(bits);
  const int passes = (bits + rb - 1) / rb;
  if (passes == 0) {
    if (vals_in_is_iota) k_iota<<<1024, 256, 0, s>>>(vals[0], n);
    return 0;
  }
  return rb == 9 ? sort_passes<K, 9>(keys, vals, n, passes, vals_in_is_iota, temp, s)
                 : sort_passes<K, 8>(keys, vals, n, passes, vals_in_is_iota, temp, s);
}

template int radix_sort_pairs<uint32_t>(uint32_t* [2], uint32_t* [2], int64_t, int, bool, void*,
                                        cudaStream_t);
template int radix_sort_pairs<unsigned long long>(unsigned long long* [2], uint32_t* [2], int64_t,
                                                  int, bool, void*, cudaStream_t);

}  // namespace gdprim
