// gd_oracle.cpp -- CPU restatement of the exact DBSCAN that the reference uses as
// ground truth (cpu-dbscan/dbscan_rtree_exp.cpp), extended from 2D to 3D.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/, the smoke()
// entry point and bench.py's cpu_baseline / reference legs may load it.  The
// product (libgbdbscan.so) never links or calls it.
//
// Semantics restated (file:line in the reference project):
//   * neighbour predicate, centre p, candidate q -- the R-tree query box
//     [p-eps, p+eps] with inclusive overlap (dbscan_rtree_exp.cpp:423-427,
//     Rtree.h:1573-1588) AND the float64 distance
//     fl(fl(dx*dx) + fl(dy*dy)) <= fl(eps*eps), dx = fl(p - q)
//     (dbscan_rtree_exp.cpp:351-358, 431-432); in 3D the third square is added
//     last, left to right.  Built with -ffp-contract=off so no FMA changes bits.
//   * core point: |N(p)| >= minPts, N(p) includes p itself (:367-373).
//   * clusters are numbered in the order of their smallest core point index,
//     because the sequential scan (:363-376) opens a cluster at the first
//     unvisited core point.
//   * a border point takes the smallest-numbered cluster whose core point has it
//     in its neighbourhood (earlier clusters expand fully first; noise is
//     relabelled at :385-388).
//   * noise keeps -1 in the reference; here it is reported as NOISE = -2
//     (common.h:8) and clusters as 0..K-1 (reference id k -> k-1).
//
// Method (not the reference's: a grid instead of an R-tree, same answers):
//   cells of side g = eps / (sqrt(d) (1 + 2^-12)): two points in one cell are
//   always neighbours, and every neighbour lies within +-2 cells per axis.
//   Core flags: count over the 5^d stencil with early exit (OpenMP).
//   Components: union-find over cells; two cells join when a core-core pair is
//   a neighbour in BOTH directions.  A pair that is a neighbour in one direction
//   only (possible only when the box test and the distance test disagree at the
//   last bit) makes the result depend on visiting order; if one is seen, the
//   labels are recomputed with the reference's sequential expansion (exact).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int32_t kNoise = -2;

struct Oracle {
  int d = 2;
  int64_t n = 0;
  double eps = 0, eps2 = 0, g = 0;
  double o[3] = {0, 0, 0};
  int64_t G[3] = {1, 1, 1};
  const double* pts = nullptr;
  std::vector<uint64_t> ukey;      // sorted unique cell keys
  std::vector<int64_t> ustart;     // start offsets into order[], size M+1
  std::vector<int64_t> order;      // point ids sorted by (cell key, id)
  std::vector<int64_t> cell_of;    // per point id: cell index
  std::vector<int64_t> cc[3];      // per cell: integer cell coordinates

  const double* P(int64_t i) const { return pts + i * d; }

  bool box_ok(const double* p, const double* q) const {
    for (int k = 0; k < d; ++k) {
      double lo = p[k] - eps;
      double hi = p[k] + eps;
      if (lo > q[k] || q[k] > hi) return false;
    }
    return true;
  }
  double dist2(const double* c, const double* q) const {
    double a = c[0] - q[0];
    double s = a * a;
    double b = c[1] - q[1];
    double t = b * b;
    s = s + t;
    if (d == 3) {
      double e = c[2] - q[2];
      double u = e * e;
      s = s + u;
    }
    return s;
  }
  bool pred(const double* c, const double* q) const {
    return box_ok(c, q) && dist2(c, q) <= eps2;
  }

  int64_t find_cell(int64_t cx, int64_t cy, int64_t cz) const {
    if (cx < 0 || cx >= G[0] || cy < 0 || cy >= G[1]) return -1;
    if (d == 3 && (cz < 0 || cz >= G[2])) return -1;
    uint64_t key = (uint64_t)cx * (uint64_t)G[1] + (uint64_t)cy;
    if (d == 3) key = key * (uint64_t)G[2] + (uint64_t)cz;
    auto it = std::lower_bound(ukey.begin(), ukey.end(), key);
    if (it == ukey.end() || *it != key) return -1;
    return (int64_t)(it - ukey.begin());
  }

  // neighbour cell list of cell c (including c), ascending offset distance
  void stencil(int64_t c, std::vector<int64_t>& out) const {
    out.clear();
    int64_t x = cc[0][c], y = cc[1][c], z = d == 3 ? cc[2][c] : 0;
    int zr = d == 3 ? 2 : 0;
    for (int dx = -2; dx <= 2; ++dx)
      for (int dy = -2; dy <= 2; ++dy)
        for (int dz = -zr; dz <= zr; ++dz) {
          int64_t b = find_cell(x + dx, y + dy, z + dz);
          if (b >= 0) out.push_back(b);
        }
  }
};

struct DSU {
  std::vector<int64_t> p;
  explicit DSU(int64_t m) : p(m) { for (int64_t i = 0; i < m; ++i) p[i] = i; }
  int64_t find(int64_t x) {
    while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
    return x;
  }
  void unite(int64_t a, int64_t b) {
    a = find(a); b = find(b);
    if (a == b) return;
    if (a < b) p[b] = a; else p[a] = b;
  }
};

}  // namespace

extern "C" {

// Returns 0 on success, 1 bad arguments, 2 grid too large, 3 non-finite input.
// counters (may be null), int64[8]:
//   0 clusters, 1 noise, 2 core, 3 border, 4 one-directional core pairs seen,
//   5 sequential re-labelling used (0/1), 6 predicate evaluations, 7 cells
int gd_oracle_dbscan(const double* pts, int64_t n, int dim, double eps, int minpts,
                     int nthreads, int32_t* labels, uint8_t* is_core, int64_t* counters) {
  if (n < 0 || (dim != 2 && dim != 3) || !(eps > 0) || !std::isfinite(eps) || minpts < 1)
    return 1;
  if (counters) std::memset(counters, 0, 8 * sizeof(int64_t));
  if (n == 0) return 0;
  if (!pts || !labels) return 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  Oracle O;
  O.d = dim; O.n = n; O.pts = pts; O.eps = eps; O.eps2 = eps * eps;
  O.g = eps / (std::sqrt((double)dim) * (1.0 + std::ldexp(1.0, -12)));
  double hi[3];
  for (int k = 0; k < dim; ++k) { O.o[k] = pts[k]; hi[k] = pts[k]; }
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < dim; ++k) {
      double v = pts[i * dim + k];
      if (!std::isfinite(v)) return 3;
      if (v < O.o[k]) O.o[k] = v;
      if (v > hi[k]) hi[k] = v;
    }
  double total = 1.0;
  for (int k = 0; k < dim; ++k) {
    double cells = std::floor((hi[k] - O.o[k]) / O.g) + 1.0;
    if (!(cells < 4e18)) return 2;
    O.G[k] = (int64_t)cells;
    total *= cells;
  }
  if (total > 4.0e18) return 2;

  // cell keys, sort
  std::vector<uint64_t> key(n);
  std::vector<int64_t> cx(n * dim);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    uint64_t k = 0;
    for (int a = 0; a < dim; ++a) {
      int64_t c = (int64_t)std::floor((pts[i * dim + a] - O.o[a]) / O.g);
      if (c < 0) c = 0;
      if (c >= O.G[a]) c = O.G[a] - 1;
      cx[i * dim + a] = c;
      k = k * (uint64_t)O.G[a] + (uint64_t)c;
    }
    key[i] = k;
  }
  O.order.resize(n);
  for (int64_t i = 0; i < n; ++i) O.order[i] = i;
  std::sort(O.order.begin(), O.order.end(), [&](int64_t a, int64_t b) {
    return key[a] < key[b] || (key[a] == key[b] && a < b);
  });
  O.cell_of.resize(n);
  for (int64_t r = 0; r < n; ++r) {
    int64_t i = O.order[r];
    if (r == 0 || key[i] != O.ukey.back()) {
      O.ukey.push_back(key[i]);
      O.ustart.push_back(r);
      for (int a = 0; a < dim; ++a) O.cc[a].push_back(cx[i * dim + a]);
    }
    O.cell_of[i] = (int64_t)O.ukey.size() - 1;
  }
  const int64_t M = (int64_t)O.ukey.size();
  O.ustart.push_back(n);
  std::vector<uint8_t> core(n, 0);
  std::atomic<int64_t> tests{0};

  // core flags
#pragma omp parallel
  {
    std::vector<int64_t> st;
    int64_t local_tests = 0;
#pragma omp for schedule(dynamic, 64)
    for (int64_t c = 0; c < M; ++c) {
      int64_t b = O.ustart[c], e = O.ustart[c + 1];
      if (e - b >= minpts) {
        for (int64_t r = b; r < e; ++r) core[O.order[r]] = 1;
        continue;
      }
      O.stencil(c, st);
      for (int64_t r = b; r < e; ++r) {
        int64_t i = O.order[r];
        const double* p = O.P(i);
        int64_t cnt = 0;
        for (size_t s = 0; s < st.size() && cnt < minpts; ++s) {
          for (int64_t rr = O.ustart[st[s]]; rr < O.ustart[st[s] + 1]; ++rr) {
            ++local_tests;
            if (O.pred(p, O.P(O.order[rr])) && ++cnt >= minpts) break;
          }
        }
        core[i] = cnt >= minpts;
      }
    }
    tests += local_tests;
  }

  // per-cell list of core members
  std::vector<int64_t> ncore(M, 0);
  for (int64_t c = 0; c < M; ++c)
    for (int64_t r = O.ustart[c]; r < O.ustart[c + 1]; ++r) ncore[c] += core[O.order[r]];

  // components over cells: pass 0 = offsets within +-1, pass 1 = the rest
  DSU dsu(M);
  int64_t asym = 0;
  {
    std::vector<int64_t> coreA, coreB;
    int zr = dim == 3 ? 2 : 0;
    for (int pass = 0; pass < 2; ++pass) {
      for (int64_t a = 0; a < M; ++a) {
        if (!ncore[a]) continue;
        coreA.clear();
        for (int64_t r = O.ustart[a]; r < O.ustart[a + 1]; ++r)
          if (core[O.order[r]]) coreA.push_back(O.order[r]);
        int64_t x = O.cc[0][a], y = O.cc[1][a], z = dim == 3 ? O.cc[2][a] : 0;
        for (int dx = -2; dx <= 2; ++dx)
          for (int dy = -2; dy <= 2; ++dy)
            for (int dz = -zr; dz <= zr; ++dz) {
              bool near = std::abs(dx) <= 1 && std::abs(dy) <= 1 && std::abs(dz) <= 1;
              if ((pass == 0) != near) continue;
              int64_t bcell = O.find_cell(x + dx, y + dy, z + dz);
              if (bcell <= a || !ncore[bcell]) continue;
              if (dsu.find(a) == dsu.find(bcell)) continue;
              coreB.clear();
              for (int64_t r = O.ustart[bcell]; r < O.ustart[bcell + 1]; ++r)
                if (core[O.order[r]]) coreB.push_back(O.order[r]);
              bool joined = false;
              for (size_t i = 0; i < coreA.size() && !joined; ++i) {
                const double* p = O.P(coreA[i]);
                for (size_t j = 0; j < coreB.size(); ++j) {
                  const double* q = O.P(coreB[j]);
                  ++tests;
                  if (!(O.dist2(p, q) <= O.eps2)) continue;
                  bool f = O.box_ok(p, q), bw = O.box_ok(q, p);
                  if (f && bw) { joined = true; break; }
                  if (f != bw) ++asym;
                }
              }
              if (joined) dsu.unite(a, bcell);
            }
      }
    }
  }

  // cluster ids by smallest core index
  std::vector<int32_t> cid(M, -1);
  int32_t K = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (!core[i]) continue;
    int64_t r = dsu.find(O.cell_of[i]);
    if (cid[r] < 0) cid[r] = K++;
  }
  // labels: core -> its cluster; border -> smallest adjacent cluster; else noise
#pragma omp parallel
  {
    std::vector<int64_t> st;
    int64_t local_tests = 0;
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
      int64_t c = O.cell_of[i];
      if (core[i]) { labels[i] = cid[dsu.find(c)]; continue; }
      int32_t best = INT32_MAX;
      O.stencil(c, st);
      const double* b = O.P(i);
      for (size_t s = 0; s < st.size(); ++s) {
        int64_t bc = st[s];
        if (!ncore[bc]) continue;
        int32_t cl = cid[dsu.find(bc)];
        if (cl >= best) continue;
        for (int64_t rr = O.ustart[bc]; rr < O.ustart[bc + 1]; ++rr) {
          int64_t j = O.order[rr];
          if (!core[j]) continue;
          ++local_tests;
          if (O.pred(O.P(j), b)) { best = cl; break; }
        }
      }
      labels[i] = best == INT32_MAX ? kNoise : best;
    }
    tests += local_tests;
  }

  int used_seq = 0;
  if (asym > 0) {
    // The reference's sequential expansion, verbatim in meaning.
    used_seq = 1;
    std::vector<int32_t> lab(n, 0);
    std::vector<int64_t> queue, st;
    int32_t cluster = 0;
    for (int64_t i = 0; i < n; ++i) {
      if (lab[i] != 0) continue;
      if (!core[i]) { lab[i] = -1; continue; }
      ++cluster;
      lab[i] = cluster;
      queue.clear();
      queue.push_back(i);
      for (size_t h = 0; h < queue.size(); ++h) {
        int64_t c = queue[h];
        const double* p = O.P(c);
        O.stencil(O.cell_of[c], st);
        for (int64_t bc : st)
          for (int64_t rr = O.ustart[bc]; rr < O.ustart[bc + 1]; ++rr) {
            int64_t q = O.order[rr];
            if (q == c || !O.pred(p, O.P(q))) continue;
            if (lab[q] == -1) { lab[q] = cluster; continue; }
            if (lab[q] != 0) continue;
            lab[q] = cluster;
            if (core[q]) queue.push_back(q);
          }
      }
    }
    for (int64_t i = 0; i < n; ++i) labels[i] = lab[i] == -1 ? kNoise : lab[i] - 1;
    K = cluster;
  }

  int64_t noise = 0, ncores = 0;
  for (int64_t i = 0; i < n; ++i) {
    noise += labels[i] == kNoise;
    ncores += core[i];
    if (is_core) is_core[i] = core[i];
  }
  if (counters) {
    counters[0] = K;
    counters[1] = noise;
    counters[2] = ncores;
    counters[3] = n - noise - ncores;
    counters[4] = asym;
    counters[5] = used_seq;
    counters[6] = tests.load();
    counters[7] = M;
  }
  return 0;
}

// The neighbour predicate alone (centre c, candidate q), for tests.
int gd_oracle_pred(const double* c, const double* q, int dim, double eps) {
  Oracle O;
  O.d = dim; O.eps = eps; O.eps2 = eps * eps;
  return O.pred(c, q) ? 1 : 0;
}

}  // extern "C"
