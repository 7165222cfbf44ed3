// gd_main.cpp -- command-line driver, the drop-in for the reference's main.exe
// (main.cu:35-459).
//
//   gbdbscan_main <dataset> [--eps E] [--minpts M] [--dim D] [--count N]
//                 [--config common.h] [--precision fp64|fp32band] [--out PATH]
//
// Same positional usage as `./main.exe <dataset.csv>` (main.cu:39-45).  The
// reference takes EPS, MINPTS, DIMENSION and DATASET_COUNT from common.h at
// compile time; here they are read at run time from a common.h-style file
// (--config, "#define NAME value" lines) and/or flags, defaulting to the values
// the reference ships (DIMENSION 2, MINPTS 3, EPS 1.5, no point limit).
// Prints the reference's summary lines (main.cu:412-432) and writes one label
// per point to ./out/cuda_dclust_extended.txt (the reference writes its sorted
// unique labels there, dbscan.cu:242-247).
#include <sys/stat.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "gbdbscan.h"

namespace {

struct Config {
  double eps = 1.5;
  int minpts = 3;
  int dim = 2;
  long long count = 0;
  int precision = GD_PREC_FP64;
  std::string out = "./out/cuda_dclust_extended.txt";
};

bool read_config(const char* path, Config& c) {
  std::ifstream f(path);
  if (!f) return false;
  std::string line;
  while (std::getline(f, line)) {
    char name[64];
    char val[64];
    if (sscanf(line.c_str(), " #define %63s %63s", name, val) != 2) continue;
    if (!strcmp(name, "EPS")) c.eps = atof(val);
    else if (!strcmp(name, "MINPTS")) c.minpts = atoi(val);
    else if (!strcmp(name, "DIMENSION")) c.dim = atoi(val);
    else if (!strcmp(name, "DATASET_COUNT")) c.count = atoll(val);
  }
  return true;
}

void usage() {
  fprintf(stderr,
          "usage: gbdbscan_main <dataset> [--eps E] [--minpts M] [--dim 2|3] [--count N]\n"
          "                     [--config common.h] [--precision fp64|fp32band] [--out PATH]\n");
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "Please provide the dataset file path in the arguments\n");
    usage();
    return 2;
  }
  Config cfg;
  const char* dataset = nullptr;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&](void) -> const char* {
      if (i + 1 >= argc) { usage(); exit(2); }
      return argv[++i];
    };
    if (a == "--eps") cfg.eps = atof(next());
    else if (a == "--minpts") cfg.minpts = atoi(next());
    else if (a == "--dim") cfg.dim = atoi(next());
    else if (a == "--count") cfg.count = atoll(next());
    else if (a == "--out") cfg.out = next();
    else if (a == "--precision") {
      std::string p = next();
      cfg.precision = p == "fp32band" ? GD_PREC_FP32_BAND : GD_PREC_FP64;
    } else if (a == "--config") {
      const char* p = next();
      if (!read_config(p, cfg)) { fprintf(stderr, "cannot read config %s\n", p); return 2; }
    } else if (a == "-h" || a == "--help") { usage(); return 0; }
    else if (!dataset) dataset = argv[i];
    else { usage(); return 2; }
  }
  if (!dataset) { usage(); return 2; }
  printf("Using dataset file %s\n", dataset);
  double* pts = nullptr;
  int64_t n = 0;
  gd_status s = gd_import_dataset(dataset, cfg.dim, cfg.count, &pts, &n);
  if (s != GD_OK) {
    printf("\nError importing the dataset: %s\n", gd_last_error());
    return 1;
  }
  for (int i = 0; i < cfg.dim && n > 0; ++i) printf("Sample Data %lf\n", pts[i]);
  printf("Preprocessed %lld data in dataset\n", (long long)n);

  gd_ctx* ctx = nullptr;
  if ((s = gd_ctx_create(0, &ctx)) != GD_OK) {
    fprintf(stderr, "%s: %s\n", gd_status_string(s), gd_last_error());
    gd_free(pts);
    return 1;
  }
  gd_ctx_set_precision(ctx, cfg.precision);
  std::vector<int32_t> labels((size_t)n);
  gd_points P{pts, n, cfg.dim, 0};
  auto t0 = std::chrono::steady_clock::now();
  s = gd_index_build(ctx, &P, cfg.eps);
  if (s == GD_OK) s = gd_expand(ctx, cfg.minpts);
  int64_t clusters = 0, noise = 0;
  if (s == GD_OK) s = gd_get_result(ctx, labels.data(), nullptr, 0, &clusters, &noise);
  auto t1 = std::chrono::steady_clock::now();
  if (s != GD_OK) {
    fprintf(stderr, "%s: %s\n", gd_status_string(s), gd_last_error());
    gd_ctx_destroy(ctx);
    gd_free(pts);
    return 1;
  }
  gd_stats st;
  gd_get_stats(ctx, &st);
  printf("==============================================\n");
  printf("DBSCAN completed. Calculating clusters...\n");
  printf("==============================================\n");
  printf("Final cluster after merging: %lld\n", (long long)clusters);
  printf("Number of noises: %lld\n", (long long)noise);
  printf("==============================================\n");
  printf("Indexing Time: %3.2f seconds\n", st.ms_index / 1e3);
  printf("Merge Time: %3.2f seconds\n", st.ms_union / 1e3);
  printf("New Seed Fill Time: %3.2f seconds\n", 0.0);
  printf("DBSCAN kernel Time: %3.2f seconds\n", (st.ms_core + st.ms_label) / 1e3);
  printf("Communication Time: %3.2f seconds\n", (st.ms_h2d + st.ms_d2h) / 1e3);
  printf("Total Time: %3.2f seconds\n", std::chrono::duration<double>(t1 - t0).count());
  printf("==============================================\n");
  std::string dir = cfg.out.substr(0, cfg.out.find_last_of('/'));
  if (!dir.empty() && dir != cfg.out) mkdir(dir.c_str(), 0755);
  if ((s = gd_write_labels(cfg.out.c_str(), labels.data(), n)) != GD_OK)
    fprintf(stderr, "%s\n", gd_last_error());
  gd_ctx_destroy(ctx);
  gd_free(pts);
  return s == GD_OK ? 0 : 1;
}
