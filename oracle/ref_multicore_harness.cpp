// ref_multicore_harness.cpp -- wraps the reference's multicore CPU DBSCAN
// (multicore-cpu/dbscan.cpp with its report.c and read_dataset.c, compiled from
// where they lie in the reference checkout) behind one C entry point, so the
// baseline it stands for can be timed on the same synthetic inputs.
//
// TIMING INFRASTRUCTURE ONLY (see oracle/build.py; output goes to oracle/_ref/).
// Its labels are not compared with anything: the program counts neighbours
// without the point itself and tests float32 sqrt(d2) <= eps, other semantics
// than the exact DBSCAN this project reproduces, and it keeps its labels local
// to its expansion routine; it reports the number of clusters it found.
//
// The program runs hard-coded dataset sweeps from main() and sets 16 OpenMP
// threads inside its neighbour scan, so this translation unit renames that
// main() out of the way and routes the thread-count call to a value the caller
// chooses (at most 16, the size of the program's per-thread counter array).
// Nothing else changes: the O(n^2) scan and the expansion are the reference's.
#include <omp.h>

static int g_gd_mc_threads = 16;
#define omp_set_num_threads(x) (omp_set_num_threads)(g_gd_mc_threads)
#define main gd_ref_multicore_program_main
#include "dbscan.cpp"
#undef main
#undef omp_set_num_threads

extern "C" {

// points: n x 2 float64, row-major (converted to the program's float pairs).
// Returns the number of clusters the program reports.
int gd_ref_multicore_dbscan(const double* pts, int n, double eps, int minpts, int threads) {
  g_gd_mc_threads = threads < 1 ? 1 : (threads > 16 ? 16 : threads);
  point* data = new point[n > 0 ? n : 1];
  for (int i = 0; i < n; ++i) {
    data[i].x = (real)pts[2 * (size_t)i];
    data[i].y = (real)pts[2 * (size_t)i + 1];
  }
  TOTAL_PTS = n;
  RADIUS = eps;
  MinPts = minpts;
  current = 0;
  initialize_report(&report[current]);
  TGPUplan plan;
  plan.device = 0;
  plan.dataN = n;
  plan.point_Data = data;
  plan.radius = (real)eps;
  plan.nOfNeighbors = &nOfNeighbors;
  plan.MinPts = minpts;
  clusterThread(plan);
  const int k = report[current].num_clusters;
  delete[] data;
  return k;
}

}  // extern "C"
