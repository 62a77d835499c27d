// tile.cuh -- shared-memory distance tiles on the FP32 CUDA cores.
//
// A CTA of 256 threads computes a (16*TQ) x 32 block of distances between
// "row" vectors (queries, or database points when assigning owners) held in
// shared memory and a tile of 32 "column" vectors (database points or
// representatives) staged by cp.async.  Thread (tq, tx) = (tid / 16, tid % 16)
// owns rows tq + 16*i (i < TQ) and columns tx + 16*j (j < 2).  Rows are stored
// with a stride of dp + 4 floats so that eight consecutive rows start in eight
// different 16-byte bank groups: the float4 loads of a quarter warp never
// conflict, and threads that share a row get a broadcast.
//
// Each distance is accumulated over dims 0..dp-1 in order, four dims per
// float4, with the reference's rounding (see rbc_common.cuh).  Dims between d
// and dp are zero in both operands and add exactly zero.
#pragma once

#include "rbc_common.cuh"

namespace rbc {

constexpr int kTileThreads = 256;
constexpr int kTileCols = 32;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(smem)), "l"(gmem));
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// Stage rows [r0, r0 + nrows) of a row-major matrix (ld floats per row, 16-byte
// aligned rows) into shared memory rows of stride S floats.  Only the first dp
// floats of each row are copied.  Rows past nrows are left untouched.
__device__ __forceinline__ void stage_rows_async(float *dst, uint32_t S, const float *src, uint64_t ld,
                                                 uint64_t r0, uint32_t nrows, uint32_t dp) {
  const uint32_t chunks = dp >> 2;
  const uint32_t total = nrows * chunks;
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    uint32_t r = t / chunks, c = t - r * chunks;
    cp_async16(dst + r * S + 4 * c, src + (r0 + r) * ld + 4 * c);
  }
}

// Same, but each row is found through an index array (gathered rows).
__device__ __forceinline__ void stage_rows_gather_async(float *dst, uint32_t S, const float *src,
                                                        uint64_t ld, const uint32_t *rows,
                                                        uint32_t nrows, uint32_t dp) {
  const uint32_t chunks = dp >> 2;
  const uint32_t total = nrows * chunks;
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    uint32_t r = t / chunks, c = t - r * chunks;
    cp_async16(dst + r * S + 4 * c, src + (uint64_t)rows[r] * ld + 4 * c);
  }
}

// Zero rows [r0, r1) of a shared-memory row block.
__device__ __forceinline__ void zero_rows(float *dst, uint32_t S, uint32_t r0, uint32_t r1, uint32_t dp) {
  const uint32_t chunks = dp >> 2;
  const uint32_t total = (r1 > r0 ? r1 - r0 : 0) * chunks;
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    uint32_t r = t / chunks, c = t - r * chunks;
    *reinterpret_cast<float4 *>(dst + (r0 + r) * S + 4 * c) = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// acc[i][j] = dist(row tq + 16 i, col tx + 16 j).
template <int METRIC, int TQ>
__device__ __forceinline__ void tile_distances(const float *__restrict__ Rs, const float *__restrict__ Cs,
                                               uint32_t S, uint32_t dp, int tq, int tx,
                                               float (&acc)[TQ][2]) {
#pragma unroll
  for (int i = 0; i < TQ; i++) {
    acc[i][0] = 0.f;
    acc[i][1] = 0.f;
  }
  const float *rp[TQ];
#pragma unroll
  for (int i = 0; i < TQ; i++) rp[i] = Rs + (tq + 16 * i) * S;
  const float *cp0 = Cs + tx * S;
  const float *cp1 = Cs + (tx + 16) * S;
#pragma unroll 2
  for (uint32_t c = 0; c < dp; c += 4) {
    float4 x0 = *reinterpret_cast<const float4 *>(cp0 + c);
    float4 x1 = *reinterpret_cast<const float4 *>(cp1 + c);
#pragma unroll
    for (int i = 0; i < TQ; i++) {
      float4 q = *reinterpret_cast<const float4 *>(rp[i] + c);
      float a0 = acc[i][0], a1 = acc[i][1];
      a0 = accum<METRIC>(a0, q.x, x0.x);
      a1 = accum<METRIC>(a1, q.x, x1.x);
      a0 = accum<METRIC>(a0, q.y, x0.y);
      a1 = accum<METRIC>(a1, q.y, x1.y);
      a0 = accum<METRIC>(a0, q.z, x0.z);
      a1 = accum<METRIC>(a1, q.z, x1.z);
      a0 = accum<METRIC>(a0, q.w, x0.w);
      a1 = accum<METRIC>(a1, q.w, x1.w);
      acc[i][0] = a0;
      acc[i][1] = a1;
    }
  }
}

}  // namespace rbc
