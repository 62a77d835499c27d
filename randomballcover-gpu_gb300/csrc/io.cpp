// io.cpp -- the reference's file formats.
//
// Input: headerless float32, row-major, rows x cols values, read row by row
// into a buffer whose rows are ld floats apart (readData, driver.cu:201-221);
// text input is whitespace-separated numbers read as double and stored as
// float (readDataText, driver.cu:224-245).  Output: all ids (uint32, k per
// row) followed by all distances (float32, k per row); the text form prints
// "%u " / "%f " per value and a newline per row (writeNeighbs,
// driver.cu:352-393).  Padding columns of the buffer are zeroed, which the
// distance kernels rely on.  The _f64 forms are the same formats with
// real = double (the reference's double build, defs.h:27-31): 8-byte values
// in the binary files, text read as double without rounding.
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/rbc_gb300.h"

namespace rbc {
int fail(int code, const std::string &msg);
}

using rbc::fail;

namespace {

template <typename T>
int read_matrix_bin(const char *what, const char *path, T *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  if (!path || (rows && !h) || ld < cols) return fail(RBC_ERR_INVALID, std::string(what) + ": bad argument");
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  for (uint64_t r = 0; r < rows; r++) {
    T *row = h + r * ld;
    size_t got = std::fread(row, sizeof(T), cols, fp);
    if (got != cols) {
      std::fclose(fp);
      return fail(RBC_ERR_IO, std::string("short read in ") + path + " at row " + std::to_string(r));
    }
    if (ld > cols) std::memset(row + cols, 0, (ld - cols) * sizeof(T));
  }
  std::fclose(fp);
  return RBC_OK;
}

template <typename T>
int read_matrix_text(const char *what, const char *path, T *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  if (!path || (rows && !h) || ld < cols) return fail(RBC_ERR_INVALID, std::string(what) + ": bad argument");
  FILE *fp = std::fopen(path, "r");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  for (uint64_t r = 0; r < rows; r++) {
    T *row = h + r * ld;
    for (uint32_t c = 0; c < cols; c++) {
      double t;
      if (std::fscanf(fp, "%lf", &t) != 1) {
        std::fclose(fp);
        return fail(RBC_ERR_IO, std::string("short read in ") + path + " at row " + std::to_string(r));
      }
      row[c] = (T)t;
    }
    if (ld > cols) std::memset(row + cols, 0, (ld - cols) * sizeof(T));
  }
  std::fclose(fp);
  return RBC_OK;
}

template <typename T>
int write_matrix_bin(const char *what, const char *path, const T *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  if (!path || (rows && !h) || ld < cols) return fail(RBC_ERR_INVALID, std::string(what) + ": bad argument");
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  for (uint64_t r = 0; r < rows; r++) {
    if (std::fwrite(h + r * ld, sizeof(T), cols, fp) != cols) {
      std::fclose(fp);
      return fail(RBC_ERR_IO, std::string("short write to ") + path);
    }
  }
  return std::fclose(fp) == 0 ? RBC_OK : fail(RBC_ERR_IO, std::string("close failed: ") + path);
}

template <typename T>
int write_neighbors_bin(const char *what, const char *path, const uint32_t *ids, const T *dists, uint64_t m,
                        uint32_t k, uint32_t ld) {
  if (!path || (m && (!ids || !dists)) || ld < k) return fail(RBC_ERR_INVALID, std::string(what) + ": bad argument");
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  bool ok = true;
  for (uint64_t i = 0; i < m && ok; i++) ok = std::fwrite(ids + i * ld, sizeof(uint32_t), k, fp) == k;
  for (uint64_t i = 0; i < m && ok; i++) ok = std::fwrite(dists + i * ld, sizeof(T), k, fp) == k;
  if (std::fclose(fp) != 0) ok = false;
  return ok ? RBC_OK : fail(RBC_ERR_IO, std::string("short write to ") + path);
}

template <typename T>
int write_neighbors_text(const char *what, const char *path, const uint32_t *ids, const T *dists, uint64_t m,
                         uint32_t k, uint32_t ld) {
  if (!path || (m && (!ids || !dists)) || ld < k) return fail(RBC_ERR_INVALID, std::string(what) + ": bad argument");
  FILE *fp = std::fopen(path, "w");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  for (uint64_t i = 0; i < m; i++) {
    for (uint32_t j = 0; j < k; j++) std::fprintf(fp, "%u ", ids[i * ld + j]);
    std::fprintf(fp, "\n");
  }
  for (uint64_t i = 0; i < m; i++) {
    for (uint32_t j = 0; j < k; j++) std::fprintf(fp, "%f ", (double)dists[i * ld + j]);
    std::fprintf(fp, "\n");
  }
  return std::fclose(fp) == 0 ? RBC_OK : fail(RBC_ERR_IO, std::string("close failed: ") + path);
}

}  // namespace

extern "C" {

int rbc_read_matrix_bin(const char *path, float *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  return read_matrix_bin("rbc_read_matrix_bin", path, h, rows, cols, ld);
}
int rbc_read_matrix_text(const char *path, float *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  return read_matrix_text("rbc_read_matrix_text", path, h, rows, cols, ld);
}
int rbc_write_matrix_bin(const char *path, const float *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  return write_matrix_bin("rbc_write_matrix_bin", path, h, rows, cols, ld);
}
int rbc_write_neighbors_bin(const char *path, const uint32_t *ids, const float *dists, uint64_t m, uint32_t k,
                            uint32_t ld) {
  return write_neighbors_bin("rbc_write_neighbors_bin", path, ids, dists, m, k, ld);
}
int rbc_write_neighbors_text(const char *path, const uint32_t *ids, const float *dists, uint64_t m, uint32_t k,
                             uint32_t ld) {
  return write_neighbors_text("rbc_write_neighbors_text", path, ids, dists, m, k, ld);
}

int rbc_read_matrix_bin_f64(const char *path, double *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  return read_matrix_bin("rbc_read_matrix_bin_f64", path, h, rows, cols, ld);
}
int rbc_read_matrix_text_f64(const char *path, double *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  return read_matrix_text("rbc_read_matrix_text_f64", path, h, rows, cols, ld);
}
int rbc_write_matrix_bin_f64(const char *path, const double *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  return write_matrix_bin("rbc_write_matrix_bin_f64", path, h, rows, cols, ld);
}
int rbc_write_neighbors_bin_f64(const char *path, const uint32_t *ids, const double *dists, uint64_t m, uint32_t k,
                                uint32_t ld) {
  return write_neighbors_bin("rbc_write_neighbors_bin_f64", path, ids, dists, m, k, ld);
}
int rbc_write_neighbors_text_f64(const char *path, const uint32_t *ids, const double *dists, uint64_t m, uint32_t k,
                                 uint32_t ld) {
  return write_neighbors_text("rbc_write_neighbors_text_f64", path, ids, dists, m, k, ld);
}

}  // extern "C"
