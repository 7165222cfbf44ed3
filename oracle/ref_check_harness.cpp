// ref_check_harness.cpp -- runs the reference's own cluster check
// (test-results/cluster-check.cpp, compiled from where it lies in the reference
// checkout) on two label files named on the command line.
//
// TEST INFRASTRUCTURE ONLY (see oracle/build.py; output goes to oracle/_ref/).
//
// The reference program reads two fixed paths and a fixed number of lines;
// this translation unit renames its main() out of the way and hands every line
// of the two named files to its comparison function,
// DetermineErrorTwoClusterResults, which prints the report.  The comparison is
// the reference's, unchanged; only its two "%f" ratios are printed with
// "%.17g" (every bit of the double) through a printf wrapper, so tests can
// compare them exactly.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <set>
#include <string>
#include <vector>

static int gd_report_printf(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  const char* f = std::strstr(fmt, "%f");
  int r;
  if (f) {
    const double v = va_arg(ap, double);
    std::string s(fmt);
    s.replace((size_t)(f - fmt), 2, "%.17g");
    r = std::printf(s.c_str(), v);
  } else {
    r = std::vprintf(fmt, ap);
  }
  va_end(ap);
  return r;
}

#define printf gd_report_printf
#define main gd_ref_cluster_check_program_main
#include "cluster-check.cpp"
#undef main
#undef printf

// one label per line, the first comma-separated field (as the reference's
// importDataset reads them)
static std::vector<int> gd_read_labels(const char* path) {
  std::vector<int> out;
  FILE* fp = std::fopen(path, "r");
  if (!fp) return out;
  char buf[4096];
  while (std::fgets(buf, sizeof buf, fp)) {
    char* field = std::strtok(buf, ",");
    int v = 0;
    if (field && std::sscanf(field, "%d", &v) == 1) out.push_back(v);
  }
  std::fclose(fp);
  return out;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: ref_cluster_check <labels_a> <labels_b>\n");
    return 2;
  }
  std::vector<int> a = gd_read_labels(argv[1]), b = gd_read_labels(argv[2]);
  DetermineErrorTwoClusterResults(&a, &b);
  std::printf("\n");
  return 0;
}
