// gd_io.cpp -- dataset and label files (host code).
//
// gd_import_dataset replaces ImportDataset (main.cu:469-498): one point per
// line, `dim` comma-separated decimal values, no header.  Unlike the reference
// it checks every row (a row with the wrong number of fields, or a field that
// is not a number, is an error naming the line) instead of reading values
// until a fixed count.  A ".f64" file is raw little-endian float64 row-major
// data (n*dim values), the fast input path for large sets.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbdbscan.h"

// gd_api.cu keeps the thread-local error message; this file reports through it.
namespace gdio {
void set_error(const std::string& m);
}

namespace {

bool ends_with(const std::string& s, const char* suf) {
  size_t n = strlen(suf);
  return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

gd_status io_fail(gd_status s, const std::string& m) {
  gdio::set_error(m);
  return s;
}

}  // namespace

extern "C" {

gd_status gd_import_dataset(const char* path, int32_t dim, int64_t max_points, double** out,
                            int64_t* n) {
  if (!path || !out || !n) return io_fail(GD_EINVAL, "gd_import_dataset: NULL argument");
  if (dim != 2 && dim != 3) return io_fail(GD_EINVAL, "gd_import_dataset: dim must be 2 or 3");
  *out = nullptr;
  *n = 0;
  FILE* fp = fopen(path, "rb");
  if (!fp) return io_fail(GD_EIO, std::string("Unable to open file ") + path);
  std::vector<char> buf;
  if (fseek(fp, 0, SEEK_END) == 0) {
    long sz = ftell(fp);
    if (sz > 0) buf.resize((size_t)sz);
    fseek(fp, 0, SEEK_SET);
  }
  size_t got = buf.empty() ? 0 : fread(buf.data(), 1, buf.size(), fp);
  fclose(fp);
  buf.resize(got);
  if (ends_with(path, ".f64")) {
    size_t vals = got / 8;
    if (got % (8 * (size_t)dim) != 0)
      return io_fail(GD_EIO, "gd_import_dataset: .f64 size is not a multiple of 8*dim");
    int64_t rows = (int64_t)(vals / dim);
    if (max_points > 0 && rows > max_points) rows = max_points;
    double* d = static_cast<double*>(malloc(sizeof(double) * (size_t)(rows > 0 ? rows * dim : 1)));
    if (!d) return io_fail(GD_ENOMEM, "gd_import_dataset: host allocation failed");
    memcpy(d, buf.data(), sizeof(double) * (size_t)rows * dim);
    *out = d;
    *n = rows;
    return GD_OK;
  }
  buf.push_back('\0');
  std::vector<double> vals;
  vals.reserve(got / 8);
  char* p = buf.data();
  char* end = p + got;
  int64_t line = 0, rows = 0;
  while (p < end && (max_points <= 0 || rows < max_points)) {
    ++line;
    char* eol = static_cast<char*>(memchr(p, '\n', (size_t)(end - p)));
    if (!eol) eol = end;
    *eol = '\0';
    // skip blank lines (incl. a lone '\r')
    char* q = p;
    while (*q == ' ' || *q == '\t' || *q == '\r') ++q;
    if (*q) {
      int fields = 0;
      while (true) {
        errno = 0;
        char* e2 = nullptr;
        double v = strtod(q, &e2);
        if (e2 == q) {
          char msg[128];
          snprintf(msg, sizeof msg, "gd_import_dataset: line %lld: field %d is not a number",
                   (long long)line, fields + 1);
          return io_fail(GD_EIO, msg);
        }
        if (fields < 3) vals.push_back(v);
        ++fields;
        q = e2;
        while (*q == ' ' || *q == '\t' || *q == '\r') ++q;
        if (*q == ',') { ++q; continue; }
        if (*q == '\0') break;
        char msg[128];
        snprintf(msg, sizeof msg, "gd_import_dataset: line %lld: unexpected character",
                 (long long)line);
        return io_fail(GD_EIO, msg);
      }
      if (fields != dim) {
        char msg[128];
        snprintf(msg, sizeof msg, "gd_import_dataset: line %lld has %d fields, expected %d",
                 (long long)line, fields, dim);
        return io_fail(GD_EIO, msg);
      }
      ++rows;
    }
    p = eol + 1;
  }
  double* d = static_cast<double*>(malloc(sizeof(double) * (vals.empty() ? 1 : vals.size())));
  if (!d) return io_fail(GD_ENOMEM, "gd_import_dataset: host allocation failed");
  if (!vals.empty()) memcpy(d, vals.data(), sizeof(double) * vals.size());
  *out = d;
  *n = rows;
  return GD_OK;
}

gd_status gd_write_labels(const char* path, const int32_t* labels, int64_t n) {
  if (!path || (n > 0 && !labels)) return io_fail(GD_EINVAL, "gd_write_labels: NULL argument");
  FILE* fp = fopen(path, "w");
  if (!fp) return io_fail(GD_EIO, std::string("Unable to open file ") + path);
  std::vector<char> buf;
  buf.reserve(1 << 20);
  char tmp[16];
  for (int64_t i = 0; i < n; ++i) {
    int len = snprintf(tmp, sizeof tmp, "%d\n", labels[i]);
    buf.insert(buf.end(), tmp, tmp + len);
    if (buf.size() > (1 << 20)) {
      fwrite(buf.data(), 1, buf.size(), fp);
      buf.clear();
    }
  }
  if (!buf.empty()) fwrite(buf.data(), 1, buf.size(), fp);
  bool ok = fclose(fp) == 0;
  return ok ? GD_OK : io_fail(GD_EIO, "gd_write_labels: write failed");
}

void gd_free(void* p) { free(p); }

}  // extern "C"
