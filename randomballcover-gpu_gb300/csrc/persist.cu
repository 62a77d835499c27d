// persist.cu -- index files: rbc_save / rbc_load.
//
// The reference keeps its rbcStruct in device memory only and rebuilds it in
// every process (rbc.cu:126-208, 363-368).  An index file lets one process
// build and others query.  Layout: a fixed 128-byte header, then the index's
// arrays in a fixed order, each written only if the index has it (the flags
// in the header say which).  All values little-endian, as in memory.  The
// tensor-core operands are not stored: loading derives them from the lists.
// A double-precision index (RBC_BUILD_F64) adds its double rows and norms.
#include <algorithm>
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

namespace rbc {

namespace {

// Byte offset and size of every array of an index file, in file order, from
// its header; checked against the file's size before anything is read.
struct FileLayout {
  uint64_t rep_ids, R, Xp, perm, offsets, radius, owner;  // offsets in the file
  uint64_t os_lists, os_counts, os_ids, os_offsets, Xo, Xi, X64, norm64, end;
};

FileLayout layout(const FileHeader &h) {
  FileLayout L{};
  const uint64_t nr = h.nr, ld = h.ld, n = h.n;
  uint64_t at = sizeof(FileHeader);
  auto take = [&at](uint64_t bytes) {
    const uint64_t o = at;
    at += bytes;
    return o;
  };
  L.rep_ids = take(nr * 4);
  L.R = take((uint64_t)pad16((uint32_t)nr) * ld * 4);
  if (h.flags & RBC_BUILD_PARTITION) {
    L.Xp = take(n * ld * 4);
    L.perm = take(n * 4);
    L.offsets = take((nr + 1) * 8);
    L.radius = take(nr * 4);
    L.owner = take(n * 4);
  }
  if (h.flags & RBC_BUILD_ONESHOT) {
    L.os_lists = take((uint64_t)pad16((uint32_t)nr) * h.lds * 4);
    L.os_counts = take(nr * 4);
    L.os_ids = take(nr * h.s * 4);
    L.os_offsets = take((nr + 1) * 8);
    L.Xo = take(nr * h.s * ld * 4);
  }
  if (h.xi_rows) L.Xi = take(h.xi_rows * ld * 4);
  if (h.flags & RBC_BUILD_F64) {
    L.X64 = take(n * h.ld64 * 8);
    L.norm64 = take(16);
  }
  L.end = at;
  return L;
}

// The header's fields against the rules every index this library writes
// follows; "" when they hold.
const char *check_header(const FileHeader &h) {
  const uint32_t known = RBC_BUILD_PARTITION | RBC_BUILD_ONESHOT | RBC_BUILD_BF16 | RBC_BUILD_F64 | kBuildKeepInput;
  if (h.n == 0 || h.n >= 0xFFFFFFFFull) return "n outside [1, 2^32-1)";
  if (h.nr == 0 || h.nr > h.n || h.nr > 32768) return "number of representatives outside [1, min(n, 32768)]";
  if (h.d == 0 || pad4(h.d) > kMaxDim) return "d outside [1, 512]";
  if (h.ld != pad16(h.d) || h.dp != pad4(h.d)) return "row strides do not match d";
  if (h.metric != RBC_L2 && h.metric != RBC_L1) return "unknown metric";
  if (h.flags & ~known) return "unknown flags";
  if (!(h.flags & (RBC_BUILD_PARTITION | RBC_BUILD_ONESHOT))) return "no lists";
  if ((h.flags & RBC_BUILD_BF16) && !(h.flags & RBC_BUILD_PARTITION)) return "tensor-core form without a partition";
  if ((h.flags & RBC_BUILD_ONESHOT) && (h.s == 0 || h.s > h.n || h.lds < h.s || h.lds % 16))
    return "one-shot list sizes";
  if (h.xi_rows && h.xi_rows != std::max<uint64_t>(pad16((uint32_t)std::min<uint64_t>(h.n, 0xFFFFFFF0ull)), h.n))
    return "padded input rows";
  if ((h.flags & RBC_BUILD_F64) && (h.ld64 < h.d || h.ld64 % 2 || h.ld64 > pad16(h.d))) return "double row stride";
  if (h.min_list > h.max_list || h.max_list > h.n) return "list length bounds";
  return "";
}

template <typename T>
bool read_at(FILE *fp, uint64_t at, std::vector<T> &v, uint64_t count) {
  v.resize(count);
  if (std::fseek(fp, (long)at, SEEK_SET) != 0) return false;
  return std::fread(v.data(), sizeof(T), count, fp) == count;
}

// The arrays that index into others, read and checked on the host: ids in
// range, list offsets increasing from 0 to the row count, the partition a
// permutation whose rows sit in the list of their owner, radii not NaN.
// "" when they hold.
struct HostArrays {
  std::vector<uint32_t> rep_ids, perm, owner, os_lists, os_counts, os_ids;
  std::vector<uint64_t> offsets, os_offsets;
  std::vector<float> radius;
};

const char *check_arrays(FILE *fp, const FileHeader &h, const FileLayout &L, HostArrays &a) {
  const uint64_t n = h.n, nr = h.nr;
  if (!read_at(fp, L.rep_ids, a.rep_ids, nr)) return "short read";
  {
    std::vector<uint32_t> sorted = a.rep_ids;
    std::sort(sorted.begin(), sorted.end());
    if (sorted.back() >= n || std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
      return "representative ids";
  }
  if (h.flags & RBC_BUILD_PARTITION) {
    if (!read_at(fp, L.perm, a.perm, n) || !read_at(fp, L.offsets, a.offsets, nr + 1) ||
        !read_at(fp, L.radius, a.radius, nr) || !read_at(fp, L.owner, a.owner, n))
      return "short read";
    if (a.offsets[0] != 0 || a.offsets[nr] != n) return "list offsets";
    uint64_t lo = UINT64_MAX, hi = 0;
    for (uint64_t r = 0; r < nr; r++) {
      if (a.offsets[r + 1] < a.offsets[r]) return "list offsets";
      lo = std::min(lo, a.offsets[r + 1] - a.offsets[r]);
      hi = std::max(hi, a.offsets[r + 1] - a.offsets[r]);
      if (!(a.radius[r] >= 0.f)) return "list radii";
    }
    if (lo != h.min_list || hi != h.max_list) return "list length bounds";
    std::vector<uint8_t> seen(n, 0);
    for (uint64_t r = 0; r < nr; r++)
      for (uint64_t p = a.offsets[r]; p < a.offsets[r + 1]; p++) {
        const uint32_t id = a.perm[p];
        if (id >= n || seen[id] || a.owner[id] != r) return "partition rows";
        seen[id] = 1;
      }
  }
  if (h.flags & RBC_BUILD_ONESHOT) {
    const uint64_t rows = pad16((uint32_t)nr);
    if (!read_at(fp, L.os_lists, a.os_lists, rows * h.lds) || !read_at(fp, L.os_counts, a.os_counts, nr) ||
        !read_at(fp, L.os_ids, a.os_ids, nr * h.s) || !read_at(fp, L.os_offsets, a.os_offsets, nr + 1))
      return "short read";
    for (uint64_t r = 0; r < nr; r++) {
      if (a.os_counts[r] > h.s) return "one-shot list counts";
      if (a.os_offsets[r] != r * h.s) return "one-shot list offsets";
      for (uint32_t j = 0; j < a.os_counts[r]; j++)
        if (a.os_lists[r * h.lds + j] >= n) return "one-shot list ids";
    }
    if (a.os_offsets[nr] != nr * h.s) return "one-shot list offsets";
    for (uint32_t id : a.os_ids)
      if (id >= n) return "one-shot list ids";
  }
  return "";
}

template <typename T>
int upload(T **dptr, const std::vector<T> &h, uint64_t &total) {
  const size_t bytes = h.size() * sizeof(T);
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(dptr), bytes ? bytes : 16);
  if (e == cudaSuccess && bytes) e = cudaMemcpy(*dptr, h.data(), bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_load: device write");
  total += bytes;
  return RBC_OK;
}

}  // namespace

}  // namespace rbc

// Every field of the header and every array that indexes into another is
// checked on the host before the first CUDA call: a damaged or foreign file
// is refused with RBC_ERR_IO and never reaches a kernel.
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
  const char *why = check_header(h);
  if (*why) return fail(RBC_ERR_IO, std::string("rbc_load: corrupt header (") + why + ")");
  const FileLayout L = layout(h);
  if (std::fseek(fp, 0, SEEK_END) != 0) return fail(RBC_ERR_IO, "rbc_load: cannot seek");
  const long size = std::ftell(fp);
  if (size < 0 || (uint64_t)size != L.end)
    return fail(RBC_ERR_IO, (uint64_t)size < L.end ? "rbc_load: truncated index file"
                                                   : "rbc_load: index file longer than its header says");
  HostArrays a;
  why = check_arrays(fp, h, L, a);
  if (*why) return fail(RBC_ERR_IO, std::string("rbc_load: corrupt index (") + why + ")");

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
  idx->rep_ids = a.rep_ids;
  std::vector<unsigned char> stage(kStage);
  const uint64_t nr = h.nr, ld = h.ld, n = h.n;
  uint64_t &tot = idx->device_bytes;
  auto bulk = [&](uint64_t at, auto **dptr, uint64_t bytes) {
    if (std::fseek(fp, (long)at, SEEK_SET) != 0) return fail(RBC_ERR_IO, "rbc_load: cannot seek");
    return read_dev(fp, dptr, bytes, stage, tot);
  };
  int rc = bulk(L.R, &idx->R, (size_t)pad16((uint32_t)nr) * ld * 4);
  if (rc == RBC_OK && (h.flags & RBC_BUILD_PARTITION)) {
    rc = bulk(L.Xp, &idx->Xp, n * ld * 4);
    if (rc == RBC_OK) rc = upload(&idx->perm, a.perm, tot);
    if (rc == RBC_OK) rc = upload(&idx->offsets, a.offsets, tot);
    if (rc == RBC_OK) rc = upload(&idx->radius, a.radius, tot);
    if (rc == RBC_OK) rc = upload(&idx->owner, a.owner, tot);
    idx->h_offsets = a.offsets;
  }
  if (rc == RBC_OK && (h.flags & RBC_BUILD_ONESHOT)) {
    rc = upload(&idx->os_lists, a.os_lists, tot);
    if (rc == RBC_OK) rc = upload(&idx->os_counts, a.os_counts, tot);
    if (rc == RBC_OK) rc = upload(&idx->os_ids, a.os_ids, tot);
    if (rc == RBC_OK) rc = upload(&idx->os_offsets, a.os_offsets, tot);
    if (rc == RBC_OK) rc = bulk(L.Xo, &idx->Xo, nr * h.s * ld * 4);
  }
  if (rc == RBC_OK && h.xi_rows) rc = bulk(L.Xi, &idx->Xi, (size_t)h.xi_rows * ld * 4);
  if (rc == RBC_OK && (h.flags & RBC_BUILD_F64)) {
    idx->ld64 = h.ld64;
    rc = bulk(L.X64, &idx->X64, n * h.ld64 * 8);
    if (rc == RBC_OK) rc = bulk(L.norm64, &idx->norm64, 16);
  }
  if (rc != RBC_OK) return rc;
  if (h.flags & RBC_BUILD_BF16) {
    rc = build_tc(idx, nullptr);
    if (rc != RBC_OK) return rc;
  }
  *out = idx;
  idx = nullptr;
  return RBC_OK;
}
