// persist.cu -- index files: rbc_save / rbc_load.
//
// The reference keeps its rbcStruct in device memory only and rebuilds it in
// every process (rbc.cu:126-208, 363-368).  An index file lets one process
// build and others query.  Layout: a fixed 128-byte header, then the index's
// arrays in a fixed order, each written only if the index has it (the flags
// in the header say which).  All values little-endian, as in memory.  The
// tensor-core operands are not stored: loading derives them from the lists.
// A double-precision index (RBC_BUILD_F64) adds its double rows and norms.
#include <cstdio>
#include <cstring>
#include <vector>

#include "engine.cuh"
#include "rbc_common.cuh"

namespace rbc {

namespace {

constexpr char kMagic[8] = {'R', 'B', 'C', 'G', 'B', '3', '0', '0'};
constexpr uint32_t kVersion = 2;

struct FileHeader {
  char magic[8];
  uint32_t version;
  uint32_t d, ld, dp, nr, s, lds, kp, flags, ld64;  // ld64: double rows (RBC_BUILD_F64)
  int32_t metric;
  uint64_t n, n_pad, xi_rows, min_list, max_list;
  uint32_t reserved[8];
};
static_assert(sizeof(FileHeader) == 128, "index file header is 128 bytes");

constexpr size_t kStage = 64u << 20;

int write_dev(FILE *fp, const void *dptr, size_t bytes, std::vector<unsigned char> &stage) {
  const unsigned char *src = static_cast<const unsigned char *>(dptr);
  for (size_t off = 0; off < bytes; off += kStage) {
    const size_t len = std::min(kStage, bytes - off);
    cudaError_t e = cudaMemcpy(stage.data(), src + off, len, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "rbc_save: device read");
    if (std::fwrite(stage.data(), 1, len, fp) != len) return fail(RBC_ERR_IO, "rbc_save: short write");
  }
  return RBC_OK;
}

template <typename T>
int read_dev(FILE *fp, T **dptr, size_t bytes, std::vector<unsigned char> &stage, uint64_t &total) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(dptr), bytes ? bytes : 16);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_load: allocation");
  total += bytes;
  unsigned char *dst = reinterpret_cast<unsigned char *>(*dptr);
  for (size_t off = 0; off < bytes; off += kStage) {
    const size_t len = std::min(kStage, bytes - off);
    if (std::fread(stage.data(), 1, len, fp) != len) return fail(RBC_ERR_IO, "rbc_load: truncated index file");
    e = cudaMemcpy(dst + off, stage.data(), len, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "rbc_load: device write");
  }
  return RBC_OK;
}

struct FileCloser {
  FILE *fp;
  ~FileCloser() {
    if (fp) std::fclose(fp);
  }
};

}  // namespace

}  // namespace rbc

using namespace rbc;

extern "C" int rbc_save(const rbc_index *idx, const char *path) {
  if (!idx || !path) return fail(RBC_ERR_INVALID, "rbc_save: NULL argument");
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(RBC_ERR_IO, std::string("rbc_save: cannot open ") + path);
  FileCloser closer{fp};
  FileHeader h{};
  std::memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.d = idx->d;
  h.ld = idx->ld;
  h.dp = idx->dp;
  h.nr = idx->nr;
  h.s = idx->s;
  h.lds = idx->lds;
  h.kp = idx->kp;
  h.flags = idx->flags;
  h.ld64 = idx->ld64;
  h.metric = idx->metric;
  h.n = idx->n;
  h.n_pad = idx->n_pad;
  h.xi_rows = idx->Xi ? idx->xi_rows : 0;
  h.min_list = idx->min_list;
  h.max_list = idx->max_list;
  if (std::fwrite(&h, sizeof(h), 1, fp) != 1) return fail(RBC_ERR_IO, "rbc_save: short write");
  if (std::fwrite(idx->rep_ids.data(), 4, idx->nr, fp) != idx->nr) return fail(RBC_ERR_IO, "rbc_save: short write");
  std::vector<unsigned char> stage(kStage);
  const uint64_t nr = idx->nr, ld = idx->ld, n = idx->n;
  int rc = write_dev(fp, idx->R, (size_t)pad16((uint32_t)nr) * ld * 4, stage);
  if (rc == RBC_OK && (idx->flags & RBC_BUILD_PARTITION)) {
    rc = write_dev(fp, idx->Xp, n * ld * 4, stage);
    if (rc == RBC_OK) rc = write_dev(fp, idx->perm, n * 4, stage);
    if (rc == RBC_OK) rc = write_dev(fp, idx->offsets, (nr + 1) * 8, stage);
    if (rc == RBC_OK) rc = write_dev(fp, idx->radius, nr * 4, stage);
    if (rc == RBC_OK) rc = write_dev(fp, idx->owner, n * 4, stage);
  }
  if (rc == RBC_OK && (idx->flags & RBC_BUILD_ONESHOT)) {
    const uint64_t total = nr * idx->s;
    rc = write_dev(fp, idx->os_lists, (size_t)pad16((uint32_t)nr) * idx->lds * 4, stage);
    if (rc == RBC_OK) rc = write_dev(fp, idx->os_counts, nr * 4, stage);
    if (rc == RBC_OK) rc = write_dev(fp, idx->os_ids, total * 4, stage);
    if (rc == RBC_OK) rc = write_dev(fp, idx->os_offsets, (nr + 1) * 8, stage);
    if (rc == RBC_OK) rc = write_dev(fp, idx->Xo, total * ld * 4, stage);
  }
  if (rc == RBC_OK && idx->Xi) rc = write_dev(fp, idx->Xi, (size_t)idx->xi_rows * ld * 4, stage);
  if (rc == RBC_OK && (idx->flags & RBC_BUILD_F64)) {
    rc = write_dev(fp, idx->X64, n * idx->ld64 * 8, stage);
    if (rc == RBC_OK) rc = write_dev(fp, idx->norm64, 16, stage);
  }
  if (rc != RBC_OK) return rc;
  FILE *f = closer.fp;
  closer.fp = nullptr;
  return std::fclose(f) == 0 ? RBC_OK : fail(RBC_ERR_IO, "rbc_save: close failed");
}

extern "C" int rbc_load(const char *path, rbc_index **out) {
  if (!path || !out) return fail(RBC_ERR_INVALID, "rbc_load: NULL argument");
  *out = nullptr;
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return fail(RBC_ERR_IO, std::string("rbc_load: cannot open ") + path);
  FileCloser closer{fp};
  FileHeader h;
  if (std::fread(&h, sizeof(h), 1, fp) != 1) return fail(RBC_ERR_IO, "rbc_load: truncated header");
  if (std::memcmp(h.magic, kMagic, 8) != 0) return fail(RBC_ERR_IO, "rbc_load: not an index file");
  if (h.version != kVersion) return fail(RBC_ERR_UNSUPPORTED, "rbc_load: unknown index file version");
  if (h.nr == 0 || h.n == 0 || h.ld < h.d || h.ld % 16) return fail(RBC_ERR_IO, "rbc_load: corrupt header");
  rbc_index *idx = new rbc_index();
  struct Guard {
    rbc_index *&i;
    ~Guard() {
      if (i) rbc_destroy(i);
    }
  } guard{idx};
  cudaError_t e = cudaGetDevice(&idx->device);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_load: cudaGetDevice");
  idx->n = h.n;
  idx->d = h.d;
  idx->ld = h.ld;
  idx->dp = h.dp;
  idx->metric = h.metric;
  idx->flags = h.flags;
  idx->nr = h.nr;
  idx->s = h.s;
  idx->lds = h.lds;
  idx->kp = h.kp;
  idx->n_pad = h.n_pad;
  idx->min_list = h.min_list;
  idx->max_list = h.max_list;
  idx->xi_rows = h.xi_rows;
  idx->rep_ids.resize(h.nr);
  if (std::fread(idx->rep_ids.data(), 4, h.nr, fp) != h.nr) return fail(RBC_ERR_IO, "rbc_load: truncated index file");
  std::vector<unsigned char> stage(kStage);
  const uint64_t nr = h.nr, ld = h.ld, n = h.n;
  uint64_t &tot = idx->device_bytes;
  int rc = read_dev(fp, &idx->R, (size_t)pad16((uint32_t)nr) * ld * 4, stage, tot);
  if (rc == RBC_OK && (h.flags & RBC_BUILD_PARTITION)) {
    rc = read_dev(fp, &idx->Xp, n * ld * 4, stage, tot);
    if (rc == RBC_OK) rc = read_dev(fp, &idx->perm, n * 4, stage, tot);
    if (rc == RBC_OK) rc = read_dev(fp, &idx->offsets, (nr + 1) * 8, stage, tot);
    if (rc == RBC_OK) rc = read_dev(fp, &idx->radius, nr * 4, stage, tot);
    if (rc == RBC_OK) rc = read_dev(fp, &idx->owner, n * 4, stage, tot);
    if (rc == RBC_OK) {
      idx->h_offsets.resize(nr + 1);
      e = cudaMemcpy(idx->h_offsets.data(), idx->offsets, (nr + 1) * 8, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) rc = cuda_fail(e, "rbc_load: offsets");
    }
  }
  if (rc == RBC_OK && (h.flags & RBC_BUILD_ONESHOT)) {
    const uint64_t total = nr * h.s;
    rc = read_dev(fp, &idx->os_lists, (size_t)pad16((uint32_t)nr) * h.lds * 4, stage, tot);
    if (rc == RBC_OK) rc = read_dev(fp, &idx->os_counts, nr * 4, stage, tot);
    if (rc == RBC_OK) rc = read_dev(fp, &idx->os_ids, total * 4, stage, tot);
    if (rc == RBC_OK) rc = read_dev(fp, &idx->os_offsets, (nr + 1) * 8, stage, tot);
    if (rc == RBC_OK) rc = read_dev(fp, &idx->Xo, total * ld * 4, stage, tot);
  }
  if (rc == RBC_OK && h.xi_rows) rc = read_dev(fp, &idx->Xi, (size_t)h.xi_rows * ld * 4, stage, tot);
  if (rc == RBC_OK && (h.flags & RBC_BUILD_F64)) {
    if (h.ld64 < h.d || h.ld64 % 2) return fail(RBC_ERR_IO, "rbc_load: corrupt header");
    idx->ld64 = h.ld64;
    rc = read_dev(fp, &idx->X64, n * h.ld64 * 8, stage, tot);
    if (rc == RBC_OK) rc = read_dev(fp, &idx->norm64, 16, stage, tot);
  }
  if (rc != RBC_OK) return rc;
  if (h.flags & RBC_BUILD_BF16) {
    if (!(h.flags & RBC_BUILD_PARTITION)) return fail(RBC_ERR_IO, "rbc_load: corrupt header");
    rc = build_tc(idx, nullptr);
    if (rc != RBC_OK) return rc;
  }
  *out = idx;
  idx = nullptr;
  return RBC_OK;
}
