// gd_check_main.cpp -- command-line label-quality report, the drop-in for the
// reference's cluster check (test-results/cluster-check.cpp).
//
//   gbdbscan_check <labels_a> <labels_b> [--count N] [--noise V]
//
// Each file holds one label per line (the first comma-separated field is read,
// as cluster-check.cpp:201-224 does).  The reference compares a fixed 10,000
// lines from fixed paths with noise = 0; here both files are named, every line
// is read unless --count limits it, and --noise sets the noise label (default
// 0, the reference's; labels written by this library use -2).  The result
// lines carry the reference's wording, so scripts that read them keep working.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbdbscan.h"

namespace {

void usage() {
  std::fprintf(stderr, "usage: gbdbscan_check <labels_a> <labels_b> [--count N] [--noise V]\n");
}

bool read_labels(const char* path, int64_t cap, std::vector<int32_t>& out) {
  FILE* fp = std::fopen(path, "r");
  if (!fp) {
    std::fprintf(stderr, "Unable to open file %s\n", path);
    return false;
  }
  char buf[4096];
  while ((cap <= 0 || (int64_t)out.size() < cap) && std::fgets(buf, sizeof buf, fp)) {
    const char* field = std::strtok(buf, ",");
    int v = 0;
    if (!field || std::sscanf(field, "%d", &v) != 1) continue;  // blank line
    out.push_back((int32_t)v);
  }
  std::fclose(fp);
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  const char* fa = nullptr;
  const char* fb = nullptr;
  int64_t count = 0;
  int32_t noise = 0;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if ((a == "--count" || a == "--noise") && i + 1 < argc) {
      if (a == "--count") count = std::atoll(argv[++i]);
      else noise = (int32_t)std::atoi(argv[++i]);
    } else if (a == "-h" || a == "--help") {
      usage();
      return 0;
    } else if (!fa) {
      fa = argv[i];
    } else if (!fb) {
      fb = argv[i];
    } else {
      usage();
      return 2;
    }
  }
  if (!fa || !fb) {
    usage();
    return 2;
  }
  std::vector<int32_t> la, lb;
  if (!read_labels(fa, count, la) || !read_labels(fb, count, lb)) return 1;
  std::printf("size of array of datapoints1: %zu, size of array of datapoints2: %zu\n", la.size(),
              lb.size());
  if (la.size() != lb.size()) {
    std::printf("ERROR: THE NUMBER OF POINTS IN EACH ARRAY ARE NOT EQUAL\n");
    return 1;
  }
  gd_label_quality q;
  const gd_status st =
      gd_label_quality_compare(la.data(), lb.data(), (int64_t)la.size(), noise, &q);
  if (st != GD_OK) {
    std::fprintf(stderr, "gbdbscan_check: %s\n", gd_last_error());
    return 1;
  }
  // the reference's count: largest label + 1 (label 0 included), at least 1
  long long ma = 0, mb = 0;
  for (int32_t v : la) ma = v > ma ? v : ma;
  for (int32_t v : lb) mb = v > mb ? v : mb;
  std::printf("num clusters in list1, list2: %lld,%lld\n", ma + 1, mb + 1);
  std::printf("distinct non-noise labels in list1, list2: %lld,%lld\n", (long long)q.clusters_a,
              (long long)q.clusters_b);
  std::printf("mismatched noise points: %lld, agreement noise points: %lld\n",
              (long long)q.noise_mismatch, (long long)q.noise_agree);
  std::printf("fraction lost due to mismatches between clusters: %f\n", q.mismatch_loss);
  std::printf("Final Error metric: %f\n", q.score);
  return 0;
}
