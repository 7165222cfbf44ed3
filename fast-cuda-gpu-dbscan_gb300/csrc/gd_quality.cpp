// gd_quality.cpp -- label-quality report: how far one labelling of a point set
// is from another (e.g. an inexact GPU DBSCAN against the exact one).
//
// The metric is the reference's cluster check (test-results/cluster-check.cpp,
// DetermineErrorTwoClusterResults, lines 41-199), restated:
//   * a point that is noise in exactly one labelling scores 0;
//   * a point that is noise in both scores 1;
//   * any other point scores the Jaccard index |A & B| / |A | B| of the two
//     clusters that hold it (A in the first labelling, B in the second);
//   * score = mean over all points ("Final Error metric"), mismatch_loss = the
//     sum of (1 - score) over points clustered in both, divided by n ("fraction
//     lost due to mismatches between clusters").
// The reference copies both clusters for every point and intersects them by
// binary search (quadratic in the cluster size); here one pass counts cluster
// sizes and the (A, B) pair sizes, so |A & B| is the pair count and |A | B| =
// |A| + |B| - |A & B|.  Per-point scores are the same double divisions of the
// same integers, summed in point order, so both sums come out bit-identical to
// the reference's.
//
// Host code only: no CUDA call, safe without a GPU.
#include <algorithm>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "gbdbscan.h"

// gd_api.cu keeps the thread-local error message; this file reports through it.
namespace gdio {
void set_error(const std::string& m);
}

namespace {

gd_status fail(gd_status s, const char* msg) {
  gdio::set_error(msg);
  return s;
}

inline uint64_t pair_key(int32_t a, int32_t b) {
  return ((uint64_t)(uint32_t)a << 32) | (uint64_t)(uint32_t)b;
}

// Points per label: a dense array over [lo, hi] when the labels span a range
// not much larger than n (the usual 0..K-1 plus noise), else a hash map.
struct LabelSizes {
  int64_t lo = 0;
  std::vector<int64_t> dense;
  std::unordered_map<int32_t, int64_t> sparse;
  bool use_dense = false;
  int64_t distinct = 0;

  void init(const int32_t* v, int64_t n, int32_t noise) {
    int64_t mn = INT64_MAX, mx = INT64_MIN;
    for (int64_t i = 0; i < n; ++i)
      if (v[i] != noise) {
        mn = std::min<int64_t>(mn, v[i]);
        mx = std::max<int64_t>(mx, v[i]);
      }
    if (mn > mx) return;  // all noise
    use_dense = mx - mn < 4 * n + 64;
    lo = mn;
    if (use_dense) dense.assign((size_t)(mx - mn + 1), 0);
    for (int64_t i = 0; i < n; ++i)
      if (v[i] != noise) {
        int64_t& c = use_dense ? dense[(size_t)(v[i] - lo)] : sparse[v[i]];
        distinct += c == 0;
        ++c;
      }
  }
  int64_t at(int32_t label) const {
    return use_dense ? dense[(size_t)(label - lo)] : sparse.find(label)->second;
  }
};

// Points per (a, b) label pair: open addressing with linear probing, grown at
// half load.
struct PairCounts {
  std::vector<uint64_t> key;
  std::vector<int64_t> cnt;
  std::vector<uint8_t> used;
  uint64_t mask = 0;
  int64_t size = 0;

  static uint64_t mix(uint64_t k) {  // splitmix64 finaliser
    k ^= k >> 30;
    k *= 0xbf58476d1ce4e5b9ull;
    k ^= k >> 27;
    k *= 0x94d049bb133111ebull;
    return k ^ (k >> 31);
  }
  void reset(uint64_t cap) {
    key.assign(cap, 0);
    cnt.assign(cap, 0);
    used.assign(cap, 0);
    mask = cap - 1;
    size = 0;
  }
  uint64_t slot(uint64_t k) const {
    uint64_t h = mix(k) & mask;
    while (used[h] && key[h] != k) h = (h + 1) & mask;
    return h;
  }
  void add(uint64_t k) {
    if (2 * (size + 1) > (int64_t)(mask + 1)) grow();
    const uint64_t h = slot(k);
    if (!used[h]) {
      used[h] = 1;
      key[h] = k;
      ++size;
    }
    ++cnt[h];
  }
  void grow() {
    std::vector<uint64_t> k0;
    std::vector<int64_t> c0;
    std::vector<uint8_t> u0;
    k0.swap(key);
    c0.swap(cnt);
    u0.swap(used);
    reset(k0.empty() ? 1024 : 2 * k0.size());
    for (size_t i = 0; i < k0.size(); ++i)
      if (u0[i]) {
        const uint64_t h = slot(k0[i]);
        used[h] = 1;
        key[h] = k0[i];
        cnt[h] = c0[i];
        ++size;
      }
  }
  int64_t at(uint64_t k) const { return cnt[slot(k)]; }
};

}  // namespace

extern "C" gd_status gd_label_quality_compare(const int32_t* a, const int32_t* b, int64_t n,
                                              int32_t noise, gd_label_quality* out) {
  if (!out) return fail(GD_EINVAL, "gd_label_quality_compare: NULL result");
  if (n < 0) return fail(GD_EINVAL, "gd_label_quality_compare: n < 0");
  if (n > 0 && (!a || !b)) return fail(GD_EINVAL, "gd_label_quality_compare: NULL labels");
  gd_label_quality q{};
  q.n = n;
  if (n == 0) {
    q.score = 1.0;  // vacuous agreement (the reference divides 0 by 0)
    *out = q;
    return GD_OK;
  }
  LabelSizes sa, sb;
  sa.init(a, n, noise);
  sb.init(b, n, noise);
  PairCounts pc;
  pc.reset(1024);
  for (int64_t i = 0; i < n; ++i)
    if (a[i] != noise && b[i] != noise) pc.add(pair_key(a[i], b[i]));
  double sum = 0.0, lost = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const bool na = a[i] == noise, nb = b[i] == noise;
    if (na != nb) {
      ++q.noise_mismatch;  // scores 0
      continue;
    }
    if (na) {
      ++q.noise_agree;
      sum += 1.0;
      continue;
    }
    const int64_t ab = pc.at(pair_key(a[i], b[i]));
    const int64_t uni = sa.at(a[i]) + sb.at(b[i]) - ab;
    const double s = ((double)ab * 1.0) / ((double)uni * 1.0);
    if (s != 1.0) lost += 1.0 - s;
    sum += s;
  }
  q.score = (1.0 * sum) / ((double)n * 1.0);
  q.mismatch_loss = lost / ((double)n * 1.0);
  q.clusters_a = sa.distinct;
  q.clusters_b = sb.distinct;
  *out = q;
  return GD_OK;
}
