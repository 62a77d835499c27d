// io.cpp -- the reference's file formats.
//
// Input: headerless float32, row-major, rows x cols values, read row by row
// into a buffer whose rows are ld floats apart (readData, driver.cu:201-221);
// text input is whitespace-separated numbers read as double and stored as
// float (readDataText, driver.cu:224-245).  Output: all ids (uint32, k per
// row) followed by all distances (float32, k per row); the text form prints
// "%u " / "%f " per value and a newline per row (writeNeighbs,
// driver.cu:352-393).  Padding columns of the buffer are zeroed, which the
// distance kernels rely on.
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/rbc_gb300.h"

namespace rbc {
int fail(int code, const std::string &msg);
}

using rbc::fail;

extern "C" {

int rbc_read_matrix_bin(const char *path, float *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  if (!path || (rows && !h) || ld < cols) return fail(RBC_ERR_INVALID, "rbc_read_matrix_bin: bad argument");
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  for (uint64_t r = 0; r < rows; r++) {
    float *row = h + r * ld;
    size_t got = std::fread(row, sizeof(float), cols, fp);
    if (got != cols) {
      std::fclose(fp);
      return fail(RBC_ERR_IO, std::string("short read in ") + path + " at row " + std::to_string(r));
    }
    if (ld > cols) std::memset(row + cols, 0, (ld - cols) * sizeof(float));
  }
  std::fclose(fp);
  return RBC_OK;
}

int rbc_read_matrix_text(const char *path, float *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  if (!path || (rows && !h) || ld < cols) return fail(RBC_ERR_INVALID, "rbc_read_matrix_text: bad argument");
  FILE *fp = std::fopen(path, "r");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  for (uint64_t r = 0; r < rows; r++) {
    float *row = h + r * ld;
    for (uint32_t c = 0; c < cols; c++) {
      double t;
      if (std::fscanf(fp, "%lf", &t) != 1) {
        std::fclose(fp);
        return fail(RBC_ERR_IO, std::string("short read in ") + path + " at row " + std::to_string(r));
      }
      row[c] = (float)t;
    }
    if (ld > cols) std::memset(row + cols, 0, (ld - cols) * sizeof(float));
  }
  std::fclose(fp);
  return RBC_OK;
}

int rbc_write_matrix_bin(const char *path, const float *h, uint64_t rows, uint32_t cols, uint32_t ld) {
  if (!path || (rows && !h) || ld < cols) return fail(RBC_ERR_INVALID, "rbc_write_matrix_bin: bad argument");
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  for (uint64_t r = 0; r < rows; r++) {
    if (std::fwrite(h + r * ld, sizeof(float), cols, fp) != cols) {
      std::fclose(fp);
      return fail(RBC_ERR_IO, std::string("short write to ") + path);
    }
  }
  return std::fclose(fp) == 0 ? RBC_OK : fail(RBC_ERR_IO, std::string("close failed: ") + path);
}

int rbc_write_neighbors_bin(const char *path, const uint32_t *ids, const float *dists, uint64_t m, uint32_t k,
                            uint32_t ld) {
  if (!path || (m && (!ids || !dists)) || ld < k) return fail(RBC_ERR_INVALID, "rbc_write_neighbors_bin: bad argument");
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  bool ok = true;
  for (uint64_t i = 0; i < m && ok; i++) ok = std::fwrite(ids + i * ld, sizeof(uint32_t), k, fp) == k;
  for (uint64_t i = 0; i < m && ok; i++) ok = std::fwrite(dists + i * ld, sizeof(float), k, fp) == k;
  if (std::fclose(fp) != 0) ok = false;
  return ok ? RBC_OK : fail(RBC_ERR_IO, std::string("short write to ") + path);
}

int rbc_write_neighbors_text(const char *path, const uint32_t *ids, const float *dists, uint64_t m, uint32_t k,
                             uint32_t ld) {
  if (!path || (m && (!ids || !dists)) || ld < k) return fail(RBC_ERR_INVALID, "rbc_write_neighbors_text: bad argument");
  FILE *fp = std::fopen(path, "w");
  if (!fp) return fail(RBC_ERR_IO, std::string("cannot open ") + path);
  for (uint64_t i = 0; i < m; i++) {
    for (uint32_t j = 0; j < k; j++) std::fprintf(fp, "%u ", ids[i * ld + j]);
    std::fprintf(fp, "\n");
  }
  for (uint64_t i = 0; i < m; i++) {
    for (uint32_t j = 0; j < k; j++) std::fprintf(fp, "%f ", dists[i * ld + j]);
    std::fprintf(fp, "\n");
  }
  return std::fclose(fp) == 0 ? RBC_OK : fail(RBC_ERR_IO, std::string("close failed: ") + path);
}

}  // extern "C"
