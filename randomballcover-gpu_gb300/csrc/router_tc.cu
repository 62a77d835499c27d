// router_tc.cu -- the router's inference on the tensor cores.
//
// Each layer of the MLP is Y = act(X W^T + b) with X (M x K) the activations
// and W (N x K) the layer's weights, both row-major with K contiguous: exactly
// the K-major operands tcgen05.mma reads.  mlp_gemm_kernel computes one
// 128 x 128 tile of Y per CTA: one thread streams 64-wide K blocks of X and W
// with TMA (128-byte swizzle) into a 3-stage ring and issues
// 128 x 128 x 16 BF16 MMAs into a tensor-memory accumulator; the four warps
// then read the accumulator rows (one TMEM lane per thread), add the bias,
// apply GELU (exact erf form, as the training kernels) and store BF16 (hidden
// layers) or FP32 (logits).  Activations between layers are BF16, so the
// logits differ from the FP32-activation training forward in low bits; they
// only choose which lists to probe first, and the search stays exact.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "engine.cuh"
#include "sm100.cuh"

namespace rbc {

namespace {

using namespace sm100;

constexpr uint32_t kGS = 3;              // pipeline stages
constexpr uint32_t kGTile = 16384;       // 128 rows x 64 BF16
constexpr size_t kGSmem = 1024 + kGS * 2 * kGTile;

template <bool GELU, bool OUT_BF16>
__global__ void __launch_bounds__(128, 1)
    mlp_gemm_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmW,
                    const float *__restrict__ bias, void *__restrict__ out, uint32_t M, uint32_t N, uint32_t ldo,
                    uint32_t KB, uint32_t *err) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[kGS], empty[kGS], done;
  __shared__ uint32_t tslot;
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t m0 = blockIdx.y * 128, n0 = blockIdx.x * 128;
  if (warp == 0) {
    tmem_alloc(&tslot, 128);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < kGS; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    fence_barrier_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;
  bool ok = true;
  if (threadIdx.x == 0) {
    prefetch_tensormap(&tmX);
    prefetch_tensormap(&tmW);
    const uint32_t idesc = idesc_bf16_f32(128, 128);
    auto load = [&](uint32_t kb) {
      const uint32_t s = kb % kGS;
      unsigned char *sa = base + s * 2 * kGTile;
      mbar_expect_tx(&full[s], 2 * kGTile);
      tma_load_2d(sa, &tmX, (int32_t)(kb * 64), (int32_t)m0, &full[s]);
      tma_load_2d(sa + kGTile, &tmW, (int32_t)(kb * 64), (int32_t)n0, &full[s]);
    };
    uint32_t issued = 0;
    for (; issued < KB && issued < kGS; issued++) load(issued);
    for (uint32_t kb = 0; kb < KB && ok; kb++) {
      const uint32_t s = kb % kGS;
      if (!(ok = mbar_wait(&full[s], (kb / kGS) & 1, err))) break;
      tc_fence_after();
      const uint32_t a0 = smem_u32(base + s * 2 * kGTile), b0 = a0 + kGTile;
#pragma unroll
      for (uint32_t kk = 0; kk < 4; kk++)
        mma_bf16(tmem, sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), idesc, (kb | kk) != 0);
      mma_commit(&empty[s]);
      // refill the previous stage once its MMAs are done (one stage of slack)
      if (kb >= 1 && issued < KB) {
        const uint32_t ps = (kb - 1) % kGS;
        if (!(ok = mbar_wait(&empty[ps], ((kb - 1) / kGS) & 1, err))) break;
        load(issued++);
      }
    }
    mma_commit(&done);
    // drain: every load issued has landed before the CTA may leave
    for (uint32_t j = 0; j < kGS && j < issued; j++) {
      const uint32_t kb = issued - 1 - j;
      mbar_wait(&full[kb % kGS], (kb / kGS) & 1, nullptr);
    }
  }
  __syncwarp();
  ok = mbar_wait(&done, 0, err);
  tc_fence_after();
  const uint32_t row = m0 + warp * 32 + lane;
#pragma unroll 1
  for (uint32_t c = 0; c < 4 && ok; c++) {
    uint32_t r[32];
    __syncwarp();
    tmem_ld32(tmem + ((warp * 32) << 16) + c * 32, r);
    tmem_wait_ld();
    const uint32_t nb = n0 + c * 32;
    if (row >= M || nb >= N) continue;
    float v[32];
#pragma unroll
    for (int j = 0; j < 32; j++) {
      const uint32_t n = nb + j;
      float t = __uint_as_float(r[j]) + (n < N ? bias[n] : 0.f);
      if (GELU) t = 0.5f * t * (1.f + erff(t * 0.70710678118654752f));
      v[j] = t;
    }
    if (OUT_BF16) {
      __nv_bfloat16 *o = reinterpret_cast<__nv_bfloat16 *>(out) + (uint64_t)row * ldo + nb;
      if (nb + 32 <= N) {
        uint32_t pk[16];
#pragma unroll
        for (int j = 0; j < 16; j++)
          pk[j] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[2 * j])) |
                  ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[2 * j + 1])) << 16);
#pragma unroll
        for (int j = 0; j < 4; j++)
          reinterpret_cast<uint4 *>(o)[j] = make_uint4(pk[4 * j], pk[4 * j + 1], pk[4 * j + 2], pk[4 * j + 3]);
      } else {
        for (uint32_t j = 0; j < 32 && nb + j < N; j++) o[j] = __float2bfloat16_rn(v[j]);
      }
    } else {
      float *o = reinterpret_cast<float *>(out) + (uint64_t)row * ldo + nb;
#pragma unroll
      for (int j = 0; j < 32; j++)
        if (nb + j < N) o[j] = v[j];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 128);
  }
}

// The last layer fused with the probe-table selection.  A CTA holds 128
// queries' hidden activations (128 x H BF16) in shared memory for the whole
// launch and streams the weights of 128 lists at a time through a 4-stage
// TMA ring; the MMA warp accumulates each block of 128 logits into one of
// two tensor-memory buffers while four epilogue warps (one query row per
// thread) read the other, add the bias and keep the K largest logits (ties
// to the lower list) in registers.  No logit is written: each query gets its
// Pn nearest representatives' lists, then the P best others.
constexpr uint32_t kTopStages = 4;
constexpr uint32_t kTopThreads = 192;  // warp 0 loads, warp 1 issues MMAs, warps 2-5 select

template <int K>
__global__ void __launch_bounds__(kTopThreads, 1)
    router_top_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmW,
                      const float *__restrict__ bias, uint32_t M, uint32_t L, uint32_t KB, uint32_t P, uint32_t Pn,
                      const uint32_t *__restrict__ nearest, const float *__restrict__ nearest_d,
                      uint32_t *__restrict__ probe, float *__restrict__ probed, uint32_t *err) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t a_full, b_full[kTopStages], b_empty[kTopStages], t_full[2], t_empty[2];
  __shared__ uint32_t tslot;
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char *sA = base, *sB = base + KB * kGTile;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t m0 = blockIdx.x * 128, nchunks = (L + 127) / 128;
  if (warp == 1) {
    tmem_alloc(&tslot, 256);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    mbar_init(&a_full, 1);
    for (uint32_t s = 0; s < kTopStages; s++) {
      mbar_init(&b_full[s], 1);
      mbar_init(&b_empty[s], 1);
    }
    for (uint32_t s = 0; s < 2; s++) {
      mbar_init(&t_full[s], 1);
      mbar_init(&t_empty[s], 4);
    }
    fence_barrier_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;
  if (warp == 0) {
    if (lane == 0) {
      prefetch_tensormap(&tmX);
      prefetch_tensormap(&tmW);
      mbar_expect_tx(&a_full, KB * kGTile);
      for (uint32_t kb = 0; kb < KB; kb++) tma_load_2d(sA + kb * kGTile, &tmX, (int32_t)(kb * 64), (int32_t)m0, &a_full);
      uint32_t it = 0;
      bool ok = true;
      for (uint32_t j = 0; j < nchunks && ok; j++)
        for (uint32_t kb = 0; kb < KB; kb++, it++) {
          const uint32_t s = it % kTopStages;
          if (it >= kTopStages && !(ok = mbar_wait(&b_empty[s], ((it / kTopStages) - 1) & 1, err))) break;
          mbar_expect_tx(&b_full[s], kGTile);
          tma_load_2d(sB + s * kGTile, &tmW, (int32_t)(kb * 64), (int32_t)(j * 128), &b_full[s]);
        }
      // drain: every load issued has landed before the CTA may leave
      mbar_wait(&a_full, 0, nullptr);
      for (uint32_t t = 0; t < kTopStages && t < it; t++) {
        const uint32_t i = it - 1 - t;
        mbar_wait(&b_full[i % kTopStages], (i / kTopStages) & 1, nullptr);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(128, 128);
      bool ok = mbar_wait(&a_full, 0, err);
      uint32_t it = 0;
      for (uint32_t j = 0; j < nchunks && ok; j++) {
        const uint32_t slot = j & 1;
        if (j >= 2 && !(ok = mbar_wait(&t_empty[slot], ((j >> 1) - 1) & 1, err))) break;
        tc_fence_after();
        for (uint32_t kb = 0; kb < KB; kb++, it++) {
          const uint32_t s = it % kTopStages;
          if (!(ok = mbar_wait(&b_full[s], (it / kTopStages) & 1, err))) break;
          tc_fence_after();
          const uint32_t a0 = smem_u32(sA + kb * kGTile), b0 = smem_u32(sB + s * kGTile);
#pragma unroll
          for (uint32_t kk = 0; kk < 4; kk++)
            mma_bf16(tmem + slot * 128, sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), idesc, (kb | kk) != 0);
          mma_commit(&b_empty[s]);
        }
        if (ok) mma_commit(&t_full[slot]);
      }
    }
  } else {
    const uint32_t ew = warp & 3, row = m0 + ew * 32 + lane;
    float tv[K];
    uint32_t ti[K];
#pragma unroll
    for (int t = 0; t < K; t++) {
      tv[t] = -INFINITY;
      ti[t] = RBC_DUMMY;
    }
    bool ok = true;
    for (uint32_t j = 0; j < nchunks && ok; j++) {
      const uint32_t slot = j & 1;
      if (!(ok = mbar_wait(&t_full[slot], (j >> 1) & 1, err))) break;
      tc_fence_after();
#pragma unroll 1
      for (uint32_t c = 0; c < 4; c++) {
        uint32_t r[32];
        __syncwarp();
        tmem_ld32(tmem + ((ew * 32) << 16) + slot * 128 + c * 32, r);
        tmem_wait_ld();
        if (c == 3) {  // the buffer's last read is in registers: it goes back to the MMA warp
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&t_empty[slot]);
        }
        const uint32_t nb = j * 128 + c * 32;
#pragma unroll
        for (int e = 0; e < 32; e++) {
          const uint32_t n = nb + e;
          if (n >= L) break;
          const float v = __uint_as_float(r[e]) + __ldg(bias + n);
          if (!(v > tv[K - 1])) continue;  // lists come in increasing order: an equal value never displaces
#pragma unroll
          for (int t = K - 1; t > 0; t--) {
            const bool shift = v > tv[t - 1];
            const bool here = !shift && v > tv[t];
            tv[t] = shift ? tv[t - 1] : (here ? v : tv[t]);
            ti[t] = shift ? ti[t - 1] : (here ? n : ti[t]);
          }
          if (v > tv[0]) {
            tv[0] = v;
            ti[0] = n;
          }
        }
      }
    }
    if (ok && row < M) {
      const uint32_t W = Pn + P;
      for (uint32_t t = 0; t < Pn; t++) {
        probe[(uint64_t)row * W + t] = nearest[(uint64_t)row * Pn + t];
        probed[(uint64_t)row * W + t] = nearest_d[(uint64_t)row * Pn + t];
      }
      uint32_t got = 0;
#pragma unroll
      for (int t = 0; t < K; t++) {
        bool taken = ti[t] == RBC_DUMMY;
        for (uint32_t u = 0; u < Pn; u++) taken |= nearest[(uint64_t)row * Pn + u] == ti[t];
        if (!taken && got < P) {
          probe[(uint64_t)row * W + Pn + got] = ti[t];
          probed[(uint64_t)row * W + Pn + got] = 0.f;
          got++;
        }
      }
      for (; got < P; got++) {
        probe[(uint64_t)row * W + Pn + got] = RBC_DUMMY;
        probed[(uint64_t)row * W + Pn + got] = 0.f;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 256);
  }
}

template <int K>
cudaError_t launch_router_top(const void *X, uint32_t M, uint32_t H, const void *W, uint32_t L, const float *bias,
                              uint32_t P, uint32_t Pn, const uint32_t *nearest, const float *nearest_d, uint32_t *probe,
                              float *probed, uint32_t *err, cudaStream_t s) {
  CUtensorMap tmX, tmW;
  cudaError_t e = tc_make_map(&tmX, X, M, H, 128);
  if (e == cudaSuccess) e = tc_make_map(&tmW, W, L, H, 128);
  const size_t smem = 1024 + (size_t)(H / 64 + kTopStages) * kGTile;
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(router_top_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  router_top_kernel<K><<<(M + 127) / 128, kTopThreads, smem, s>>>(tmX, tmW, bias, M, L, H / 64, P, Pn, nearest,
                                                                  nearest_d, probe, probed, err);
  return launched();
}

// rows x cols FP32 (row stride ld) -> rows x kp BF16, zero beyond cols.
__global__ void pad_bf16_kernel(const float *__restrict__ src, uint32_t ld, uint64_t rows, uint32_t cols,
                                uint32_t kp, __nv_bfloat16 *__restrict__ dst) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= rows * kp) return;
  const uint64_t r = i / kp;
  const uint32_t c = (uint32_t)(i - r * kp);
  dst[i] = __float2bfloat16_rn(c < cols ? src[r * ld + c] : 0.f);
}

// W1 (H x d BF16) -> H x kp BF16, zero beyond d.
__global__ void pad_w1_kernel(const __nv_bfloat16 *__restrict__ w1, uint32_t H, uint32_t d, uint32_t kp,
                              __nv_bfloat16 *__restrict__ dst) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= (uint64_t)H * kp) return;
  const uint64_t r = i / kp;
  const uint32_t c = (uint32_t)(i - r * kp);
  dst[i] = c < d ? w1[r * d + c] : __float2bfloat16_rn(0.f);
}

template <bool GELU, bool OUT_BF16>
cudaError_t gemm_tc(const void *X, uint32_t M, uint32_t K, const void *W, uint32_t N, const float *bias, void *out,
                    uint32_t ldo, uint32_t *err, cudaStream_t s) {
  CUtensorMap tmX, tmW;
  cudaError_t e = tc_make_map(&tmX, X, M, K, 128);
  if (e == cudaSuccess) e = tc_make_map(&tmW, W, N, K, 128);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(mlp_gemm_kernel<GELU, OUT_BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kGSmem);
  if (e != cudaSuccess) return e;
  dim3 grid((N + 127) / 128, (M + 127) / 128);
  mlp_gemm_kernel<GELU, OUT_BF16><<<grid, 128, kGSmem, s>>>(tmX, tmW, bias, out, M, N, ldo, K / 64, err);
  return launched();
}

}  // namespace

bool Router::tc_ok() const { return H % 64 == 0 && H >= 64; }

bool Router::top_ok(uint32_t width) const { return tc_ok() && H <= 512 && width >= 1 && width <= 16; }

cudaError_t Router::probes_tc(const float *Xin, uint32_t ldx, uint32_t b, uint32_t P, uint32_t Pn,
                              const uint32_t *nearest, const float *nearest_d, uint32_t *probe, float *probed,
                              uint32_t *err, cudaStream_t s) {
  if (!top_ok(P + Pn)) return cudaErrorInvalidValue;
  cudaError_t e = forward_tc(Xin, ldx, b, nullptr, err, s);
  if (e != cudaSuccess) return e;
  const __nv_bfloat16 *W3 = wb + (size_t)H * d + H + (size_t)H * H + H;
  const float *b3 = w + (size_t)H * d + H + (size_t)H * H + H + (size_t)(L + T) * H;
  const uint32_t width = P + Pn;
  if (width <= 2) return launch_router_top<2>(h2b, b, H, W3, L, b3, P, Pn, nearest, nearest_d, probe, probed, err, s);
  if (width <= 4) return launch_router_top<4>(h2b, b, H, W3, L, b3, P, Pn, nearest, nearest_d, probe, probed, err, s);
  if (width <= 8) return launch_router_top<8>(h2b, b, H, W3, L, b3, P, Pn, nearest, nearest_d, probe, probed, err, s);
  return launch_router_top<16>(h2b, b, H, W3, L, b3, P, Pn, nearest, nearest_d, probe, probed, err, s);
}

cudaError_t Router::forward_tc(const float *Xin, uint32_t ldx, uint32_t b, float *zout, uint32_t *err,
                               cudaStream_t s) {
  if (!tc_ok()) return cudaErrorInvalidValue;
  const uint32_t kp = (d + 63) / 64 * 64;
  cudaError_t e = cudaSuccess;
  if (b > tc_cap) {
    for (void *p : {(void *)xb, (void *)h1b, (void *)h2b})
      if (p) cudaFreeAsync(p, s);
    xb = h1b = h2b = nullptr;
    e = cudaMallocAsync((void **)&xb, (size_t)b * kp * 2, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&h1b, (size_t)b * H * 2, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&h2b, (size_t)b * H * 2, s);
    tc_cap = e == cudaSuccess ? b : 0;
    if (e != cudaSuccess) return e;
  }
  if (!w1p) {
    e = cudaMalloc((void **)&w1p, (size_t)H * kp * 2);
    if (e != cudaSuccess) return e;
  }
  if (w1p_version != version) {  // the padded W1 follows the BF16 weights
    pad_w1_kernel<<<(unsigned)(((uint64_t)H * kp + 255) / 256), 256, 0, s>>>(wb, H, d, kp, w1p);
    if ((e = launched()) != cudaSuccess) return e;
    w1p_version = version;
  }
  const __nv_bfloat16 *W2 = wb + (size_t)H * d + H, *W3 = W2 + (size_t)H * H + H;
  const float *b1 = w + (size_t)H * d, *b2 = b1 + H + (size_t)H * H, *b3 = b2 + H + (size_t)(L + T) * H;
  pad_bf16_kernel<<<(unsigned)(((uint64_t)b * kp + 255) / 256), 256, 0, s>>>(Xin, ldx, b, d, kp, xb);
  if ((e = launched()) != cudaSuccess) return e;
  if ((e = gemm_tc<true, true>(xb, b, kp, w1p, H, b1, h1b, H, err, s)) != cudaSuccess) return e;
  if ((e = gemm_tc<true, true>(h1b, b, H, W2, H, b2, h2b, H, err, s)) != cudaSuccess) return e;
  if (!zout) return cudaSuccess;  // the hidden activations alone (the distance head reads them)
  return gemm_tc<false, false>(h2b, b, H, W3, L, b3, zout, L, err, s);
}

// The distance head: zt[r] = a2[r] . W3[L] + b3[L], one warp per row over the
// BF16 activations of the tensor-core layers.
__global__ void head_kernel(const __nv_bfloat16 *__restrict__ a2, uint32_t b, uint32_t H,
                            const __nv_bfloat16 *__restrict__ wrow, const float *__restrict__ bias,
                            float *__restrict__ zt) {
  const uint64_t r = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (r >= b) return;
  float acc = 0.f;
  for (uint32_t h = lane; h < H; h += 32)
    acc = fmaf(__bfloat162float(a2[r * H + h]), __bfloat162float(wrow[h]), acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) zt[r] = acc + *bias;
}

cudaError_t Router::forward_tc_head(const float *Xin, uint32_t ldx, uint32_t b, float *zt_out, uint32_t *err,
                                    cudaStream_t s) {
  if (!T) return cudaErrorInvalidValue;
  cudaError_t e = forward_tc(Xin, ldx, b, nullptr, err, s);
  if (e != cudaSuccess) return e;
  const __nv_bfloat16 *W3 = wb + (size_t)H * d + H + (size_t)H * H + H;
  const float *b3 = w + (size_t)H * d + H + (size_t)H * H + H + (size_t)(L + T) * H;
  head_kernel<<<(unsigned)(((uint64_t)b * 32 + 255) / 256), 256, 0, s>>>(h2b, b, H, W3 + (size_t)L * H, b3 + L,
                                                                        zt_out);
  return launched();
}

}  // namespace rbc
