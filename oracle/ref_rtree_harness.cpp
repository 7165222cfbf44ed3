// ref_rtree_harness.cpp -- wraps the reference's own exact CPU DBSCAN
// (cpu-dbscan/dbscan_rtree_exp.cpp + its vendored Rtree.h, compiled from where
// they lie in the reference checkout) behind one C entry point, so tests can run
// the real reference on the same inputs as the restated oracle.
//
// TEST INFRASTRUCTURE ONLY (see oracle/build.py; output goes to oracle/_ref/).
//
// The reference program keeps its result in a private member and its main()
// runs hard-coded dataset sweeps, so this translation unit makes the members
// reachable and renames that main() out of the way.  Nothing else changes: the
// R-tree build, the neighbour query and the expansion are the reference's.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <assert.h>
#include <math.h>

#include <algorithm>
#include <ctime>
#include <fstream>
#include <functional>
#include <iostream>
#include <vector>

#define private public
#define main gd_ref_rtree_program_main
#include "dbscan_rtree_exp.cpp"
#undef main
#undef private

extern "C" {

// points: n x 2 float64, row-major.  clusters_out: the reference's labels
// (-1 noise, 1..K clusters).  Returns K.
int gd_ref_rtree_dbscan(const double* points, int n, double eps, int minpts,
                        int* clusters_out) {
  DATASET_SIZE = n;
  double** rows = (double**)malloc(sizeof(double*) * (n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) rows[i] = const_cast<double*>(points + 2 * (size_t)i);
  DBSCAN* db = new DBSCAN(rows, eps, minpts);
  db->run();
  memcpy(clusters_out, db->clusters, sizeof(int) * (size_t)n);
  int k = db->cluster;
  delete db;
  free(rows);
  return k;
}

}  // extern "C"
