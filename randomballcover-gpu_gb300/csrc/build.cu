// build.cu -- index construction kernels.
//
// Partition lists (exact search).  Each database row is assigned to its
// nearest representative (dist.cu argmin), then the row ids are stably
// counting-sorted by owner:
//   owner_hist    per tile of rows, a histogram over owners   (getCountsKernel,
//                                                               sKernel.cu:136-141)
//   exclusive_scan over the (owner, tile) histogram            (sumKernel /
//                                                               combineSumKernel,
//                                                               sKernel.cu:14-133)
//   owner_scatter row ids to their list slots, ids ascending   (buildMapKernel,
//                                                               sKernel.cu:144-153)
//   gather_rows   a contiguous list-major copy of the rows, so the query streams
//                 each list with coalesced 16-byte copies.
// The reference builds its lists from an nr x n byte mask; at n = 10M that
// matrix cannot exist, while the tile histogram here is nr x n/8192 words.
//
// One-shot lists (the reference's build, rbc.cu:126-208).  For a block of
// representatives the distance block is computed (dist.cu dense), then per row
//   row_select    the exact s-th smallest distance by a 3-pass radix select on
//                 the float bit patterns (replaces the bisection of
//                 findRangeKernel, kernels.cu:322-414, which has no iteration
//                 bound and yields "about s" points), and
//   row_compact   mask + scan + scatter + count fused into one pass per row
//                 (rangeSearchKernel, sumKernel, buildMapKernel,
//                 getCountsKernel): exactly min(s, n) ids per list, ties at the
//                 threshold to the lower ids, stored in increasing id order.
#include <algorithm>

#include "kernels.cuh"
#include "rbc_common.cuh"

namespace rbc {

namespace {

constexpr uint32_t kOwnerTile = 8192;  // rows per histogram tile

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------------- layouts
__global__ void pad_rows_kernel(const float *__restrict__ src, uint64_t ld_src, float *__restrict__ dst,
                                uint32_t ld_dst, uint64_t rows, uint32_t d) {
  uint64_t total = rows * ld_dst;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t r = i / ld_dst;
    uint32_t c = (uint32_t)(i - r * ld_dst);
    dst[i] = c < d ? src[r * ld_src + c] : 0.f;
  }
}

__global__ void gather_rows_kernel(const float4 *__restrict__ src, uint32_t ld4,
                                   const uint32_t *__restrict__ rows, uint64_t n, float4 *__restrict__ dst) {
  uint64_t total = n * ld4;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t r = i / ld4;
    uint32_t c = (uint32_t)(i - r * ld4);
    dst[i] = __ldg(src + (uint64_t)rows[r] * ld4 + c);
  }
}

// ---------------------------------------------------------------- partition
// One warp per tile: rows are visited in increasing order 32 at a time, so the
// per-owner counts (and, in the scatter, the slots) follow the row order.
__global__ void owner_hist_kernel(const uint32_t *__restrict__ owner, uint64_t n, uint32_t nr,
                                  uint32_t *__restrict__ hist, uint32_t ntiles) {
  extern __shared__ uint32_t h[];
  const uint32_t tile = blockIdx.x, lane = threadIdx.x;
  for (uint32_t r = lane; r < nr; r += 32) h[r] = 0;
  __syncwarp();
  const uint64_t b0 = (uint64_t)tile * kOwnerTile;
  const uint64_t b1 = min(n, b0 + kOwnerTile);
  for (uint64_t b = b0; b < b1; b += 32) {
    uint64_t i = b + lane;
    bool v = i < b1;
    uint32_t act = __ballot_sync(0xffffffffu, v);
    if (v) {
      uint32_t o = owner[i];
      uint32_t peers = __match_any_sync(act, o);
      if ((peers & lanemask_lt()) == 0) h[o] += __popc(peers);
    }
    __syncwarp();
  }
  for (uint32_t r = lane; r < nr; r += 32) hist[(uint64_t)r * ntiles + tile] = h[r];
}

__global__ void owner_scatter_kernel(const uint32_t *__restrict__ owner, uint64_t n, uint32_t nr,
                                     const uint32_t *__restrict__ scan, uint32_t ntiles,
                                     uint32_t *__restrict__ perm) {
  extern __shared__ uint32_t cur[];
  const uint32_t tile = blockIdx.x, lane = threadIdx.x;
  for (uint32_t r = lane; r < nr; r += 32) cur[r] = scan[(uint64_t)r * ntiles + tile];
  __syncwarp();
  const uint64_t b0 = (uint64_t)tile * kOwnerTile;
  const uint64_t b1 = min(n, b0 + kOwnerTile);
  for (uint64_t b = b0; b < b1; b += 32) {
    uint64_t i = b + lane;
    bool v = i < b1;
    uint32_t act = __ballot_sync(0xffffffffu, v);
    uint32_t o = 0, peers = 0, base = 0;
    if (v) {
      o = owner[i];
      peers = __match_any_sync(act, o);
      base = cur[o];
      perm[base + __popc(peers & lanemask_lt())] = (uint32_t)i;
    }
    __syncwarp();
    if (v && (peers & lanemask_lt()) == 0) cur[o] = base + __popc(peers);
    __syncwarp();
  }
}

__global__ void list_offsets_kernel(const uint32_t *__restrict__ scan, uint32_t nr, uint32_t ntiles,
                                    uint64_t n, uint64_t *__restrict__ offsets) {
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nr) offsets[r] = scan[(uint64_t)r * ntiles];
  if (r == nr) offsets[nr] = n;
}

// radius[r] = largest owner distance among the members of list r (one warp per list).
__global__ void list_radius_kernel(const uint64_t *__restrict__ offsets, const uint32_t *__restrict__ perm,
                                   const float *__restrict__ odist, uint32_t nr, float *__restrict__ radius) {
  uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= nr) return;
  float mx = 0.f;
  for (uint64_t p = offsets[w] + lane; p < offsets[w + 1]; p += 32) mx = fmaxf(mx, odist[perm[p]]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) radius[w] = mx;
}

// ---------------------------------------------------------------- scan
// Reduce-then-scan in three launches per level (no inter-CTA waiting).
constexpr uint32_t kScanThreads = 256, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_sums, uint32_t &total) {
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) warp_sums[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t s = lane < blockDim.x / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= (uint32_t)o) s += y;
    }
    warp_sums[lane] = s;  // inclusive
  }
  __syncthreads();
  total = warp_sums[blockDim.x / 32 - 1];
  uint32_t before = w ? warp_sums[w - 1] : 0;
  __syncthreads();
  return before + x - v;
}

__global__ void scan_reduce_kernel(const uint32_t *__restrict__ in, uint64_t n, uint32_t *__restrict__ sums) {
  __shared__ uint32_t ws[32];
  uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint32_t s = 0;
  for (uint32_t j = 0; j < kScanItems; j++) {
    uint64_t i = base + (uint64_t)j * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  uint32_t total;
  block_exclusive_scan(s, ws, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_tile_kernel(const uint32_t *__restrict__ in, uint64_t n, uint32_t *__restrict__ out,
                                 const uint32_t *__restrict__ offs) {
  __shared__ uint32_t ws[32];
  uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (uint32_t j = 0; j < kScanItems; j++) {
    uint64_t i = base + j;
    v[j] = i < n ? in[i] : 0;
    s += v[j];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan(s, ws, total) + (offs ? offs[blockIdx.x] : 0);
#pragma unroll
  for (uint32_t j = 0; j < kScanItems; j++) {
    uint64_t i = base + j;
    if (i < n) out[i] = run;
    run += v[j];
  }
}

// ---------------------------------------------------------------- one-shot select
constexpr uint32_t kSelThreads = 1024;

// Find the bin b where the running count crosses `want` (1-based) over
// `nbins` bins held in smem: sets *bin and *before (count in bins < b).
__device__ void find_bin(const uint32_t *hist, uint32_t nbins, uint32_t want, uint32_t *ws, uint32_t *bin,
                         uint32_t *before) {
  const uint32_t per = (nbins + kSelThreads - 1) / kSelThreads;
  uint32_t local = 0;
  for (uint32_t j = 0; j < per; j++) {
    uint32_t b = threadIdx.x * per + j;
    if (b < nbins) local += hist[b];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan(local, ws, total);
  for (uint32_t j = 0; j < per; j++) {
    uint32_t b = threadIdx.x * per + j;
    if (b < nbins) {
      uint32_t h = hist[b];
      if (run < want && want <= run + h) {
        *bin = b;
        *before = run;
      }
      run += h;
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kSelThreads) row_select_kernel(const float *__restrict__ D, uint64_t ldD,
                                                                 uint64_t n, uint32_t s,
                                                                 uint32_t *__restrict__ thr_bits,
                                                                 uint32_t *__restrict__ need) {
  __shared__ uint32_t hist[2048];
  __shared__ uint32_t ws[32];
  __shared__ uint32_t s_bin, s_before;
  const uint32_t *row = reinterpret_cast<const uint32_t *>(D + blockIdx.x * ldD);
  uint32_t prefix = 0, want = s;
  // passes over bits [31:21], [20:10], [9:0]
  const int shifts[3] = {21, 10, 0};
  const uint32_t widths[3] = {11, 11, 10};
  for (int p = 0; p < 3; p++) {
    const uint32_t nb = 1u << widths[p];
    for (uint32_t b = threadIdx.x; b < nb; b += kSelThreads) hist[b] = 0;
    __syncthreads();
    const int hi_shift = shifts[p] + widths[p];  // bits above this pass must equal prefix
    // 16-byte loads (ldD % 4 == 0), four values per thread and step
    const uint4 *row4 = reinterpret_cast<const uint4 *>(row);
    for (uint64_t i = 4 * (uint64_t)threadIdx.x; i < n; i += 4 * kSelThreads) {
      const uint4 q = row4[i >> 2];
      const uint32_t v[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const bool match = i + j < n && (p == 0 || (v[j] >> hi_shift) == prefix);
        if (match) atomicAdd(&hist[(v[j] >> shifts[p]) & (nb - 1)], 1u);
      }
    }
    __syncthreads();
    find_bin(hist, nb, want, ws, &s_bin, &s_before);
    prefix = (prefix << widths[p]) | s_bin;
    want -= s_before;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    thr_bits[blockIdx.x] = prefix;  // the s-th smallest value
    need[blockIdx.x] = want;        // how many of the values equal to it are taken
  }
}

// Ids of row b's selected entries, increasing: every value below the s-th
// smallest, and the first `need` values equal to it.  Each thread holds 8
// consecutive values (two 16-byte loads) per chunk of 8 x kSelThreads values;
// one block scan per chunk of the packed counts (equal values << 16 | values
// below) places every selected id, the first `need` equal ones included.
constexpr int kCompactPer = 8;
__global__ void __launch_bounds__(kSelThreads) row_compact_kernel(const float *__restrict__ D, uint64_t ldD,
                                                                  uint64_t n, const uint32_t *__restrict__ thr_bits,
                                                                  const uint32_t *__restrict__ need,
                                                                  uint32_t *__restrict__ lists, uint32_t lds,
                                                                  uint32_t *__restrict__ counts) {
  __shared__ uint32_t ws[32];
  const uint4 *row = reinterpret_cast<const uint4 *>(D + blockIdx.x * ldD);  // ldD % 4 == 0
  const uint32_t t = thr_bits[blockIdx.x], nd = need[blockIdx.x];
  uint32_t *out = lists + (uint64_t)blockIdx.x * lds;
  uint32_t taken = 0, eq_seen = 0;
  constexpr uint64_t kChunk = kCompactPer * kSelThreads;
  for (uint64_t c0 = 0; c0 < n; c0 += kChunk) {
    const uint64_t i0 = c0 + kCompactPer * threadIdx.x;
    uint32_t v[kCompactPer];
#pragma unroll
    for (int h = 0; h < kCompactPer / 4; h++) {
      const uint4 q = i0 + 4 * h < n ? row[(i0 >> 2) + h] : make_uint4(~0u, ~0u, ~0u, ~0u);
      v[4 * h] = q.x;
      v[4 * h + 1] = q.y;
      v[4 * h + 2] = q.z;
      v[4 * h + 3] = q.w;
    }
    uint32_t nlt = 0, neq = 0;
#pragma unroll
    for (int j = 0; j < kCompactPer; j++) {
      if (i0 + j >= n) v[j] = ~0u;  // above any distance's bits: never selected
      nlt += v[j] < t;
      neq += v[j] == t;
    }
    uint32_t tot;
    const uint32_t pre = block_exclusive_scan((neq << 16) | nlt, ws, tot);  // both fields < 2^16
    const uint32_t eq_left = nd > eq_seen ? nd - eq_seen : 0;  // equal values still to take
    uint32_t eq_pos = pre >> 16;
    uint32_t pos = taken + (pre & 0xFFFFu) + min(eq_pos, eq_left);
#pragma unroll
    for (int j = 0; j < kCompactPer; j++) {
      const bool eq = v[j] == t;
      if (v[j] < t || (eq && eq_pos < eq_left)) out[pos++] = (uint32_t)(i0 + j);
      eq_pos += eq;
    }
    taken += (tot & 0xFFFFu) + min(tot >> 16, eq_left);
    eq_seen += tot >> 16;
  }
  if (threadIdx.x == 0) counts[blockIdx.x] = taken;
}

}  // namespace

uint32_t owner_tile_rows() { return kOwnerTile; }

cudaError_t launch_pad_rows(const float *src, uint64_t ld_src, float *dst, uint32_t ld_dst, uint64_t rows,
                            uint32_t d, cudaStream_t s) {
  if (rows == 0) return cudaSuccess;
  uint64_t total = rows * ld_dst;
  unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, 152ull * 64);
  pad_rows_kernel<<<grid, 256, 0, s>>>(src, ld_src, dst, ld_dst, rows, d);
  return launched();
}

cudaError_t launch_gather_rows(const float *src, uint32_t ld, const uint32_t *rows, uint64_t n, float *dst,
                               cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  uint64_t total = n * (ld / 4);
  unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, 152ull * 64);
  gather_rows_kernel<<<grid, 256, 0, s>>>(reinterpret_cast<const float4 *>(src), ld / 4, rows, n,
                                          reinterpret_cast<float4 *>(dst));
  return launched();
}

cudaError_t launch_owner_hist(const uint32_t *owner, uint64_t n, uint32_t nr, uint32_t *hist, uint32_t ntiles,
                              cudaStream_t s) {
  size_t smem = (size_t)nr * 4;
  cudaError_t e = cudaFuncSetAttribute(owner_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  owner_hist_kernel<<<ntiles, 32, smem, s>>>(owner, n, nr, hist, ntiles);
  return launched();
}

cudaError_t launch_owner_scatter(const uint32_t *owner, uint64_t n, uint32_t nr, const uint32_t *hist_scan,
                                 uint32_t ntiles, uint32_t *perm, cudaStream_t s) {
  size_t smem = (size_t)nr * 4;
  cudaError_t e = cudaFuncSetAttribute(owner_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  owner_scatter_kernel<<<ntiles, 32, smem, s>>>(owner, n, nr, hist_scan, ntiles, perm);
  return launched();
}

cudaError_t launch_list_offsets(const uint32_t *hist_scan, uint32_t nr, uint32_t ntiles, uint64_t n,
                                uint64_t *offsets, cudaStream_t s) {
  list_offsets_kernel<<<(nr + 1 + 255) / 256, 256, 0, s>>>(hist_scan, nr, ntiles, n, offsets);
  return launched();
}

cudaError_t launch_list_radius(const uint64_t *offsets, const uint32_t *perm, const float *odist, uint32_t nr,
                               float *radius, cudaStream_t s) {
  unsigned grid = (unsigned)(((uint64_t)nr * 32 + 255) / 256);
  list_radius_kernel<<<grid, 256, 0, s>>>(offsets, perm, odist, nr, radius);
  return launched();
}

static uint64_t scan_blocks(uint64_t n) { return (n + kScanTile - 1) / kScanTile; }

size_t scan_temp_bytes(uint64_t n) {
  size_t bytes = 0;
  while (n > kScanTile) {
    n = scan_blocks(n);
    bytes += (size_t)(n + 64) * 4 * 2;
  }
  return bytes + 256;
}

cudaError_t launch_exclusive_scan(const uint32_t *in, uint32_t *out, uint64_t n, void *temp, uint32_t *err,
                                  cudaStream_t s) {
  (void)err;
  if (n == 0) return cudaSuccess;
  if (n <= kScanTile) {
    scan_tile_kernel<<<1, kScanThreads, 0, s>>>(in, n, out, nullptr);
    return launched();
  }
  uint64_t nb = scan_blocks(n);
  uint32_t *sums = reinterpret_cast<uint32_t *>(temp);
  uint32_t *sums_scan = sums + nb + 64;
  scan_reduce_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, sums);
  cudaError_t e = launch_exclusive_scan(sums, sums_scan, nb, sums_scan + nb + 64, err, s);
  if (e != cudaSuccess) return e;
  scan_tile_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, out, sums_scan);
  return launched();
}

cudaError_t launch_row_select(const float *D, uint64_t ldD, uint32_t rows, uint64_t n, uint32_t s,
                              uint32_t *thr_bits, uint32_t *need, cudaStream_t st) {
  if (rows == 0) return cudaSuccess;
  row_select_kernel<<<rows, kSelThreads, 0, st>>>(D, ldD, n, s, thr_bits, need);
  return launched();
}

cudaError_t launch_row_compact(const float *D, uint64_t ldD, uint32_t rows, uint64_t n, const uint32_t *thr_bits,
                               const uint32_t *need, uint32_t *lists, uint32_t lds, uint32_t *counts,
                               cudaStream_t st) {
  if (rows == 0) return cudaSuccess;
  row_compact_kernel<<<rows, kSelThreads, 0, st>>>(D, ldD, n, thr_bits, need, lists, lds, counts);
  return launched();
}

}  // namespace rbc
