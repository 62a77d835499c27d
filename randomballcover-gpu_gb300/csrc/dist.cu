// dist.cu -- dense distance tiles, nearest-row search and range counts.
//
// Counterparts of the reference's dist1Kernel (kernels.cu:285-317, the
// representative x database distance block of the build), nnKernel
// (kernels.cu:165-222, nearest representative of each query / point) and
// rangeCountKernel (kernels.cu:426-471).  All three stage a block of 16*TQ
// "row" vectors in shared memory once and stream the other operand through a
// double-buffered cp.async pipeline in tiles of 32 (tile.cuh).  Ties in the
// nearest-row search go to the lower row index, the (dist, index) order of
// bruteCPU (brute.cu:104) -- the reference's nnKernel keeps the lower thread
// slot instead, which is not an order on indices.
#include <algorithm>

#include "kernels.cuh"
#include "tile.cuh"

namespace rbc {

namespace {

template <int TQ>
size_t rows_smem_bytes(uint32_t dp) {
  uint32_t S = dp + 4;
  return ((size_t)16 * TQ * S + 2 * kTileCols * S) * 4;
}

// Stage BQ rows [r0, r0 + valid) of A (zero rows past valid).
template <int TQ>
__device__ __forceinline__ void stage_row_block(float *Rs, uint32_t S, const float *A, uint32_t ld,
                                                uint64_t r0, uint32_t valid, uint32_t dp) {
  constexpr uint32_t BQ = 16 * TQ;
  const uint32_t chunks = dp >> 2;
  for (uint32_t t = threadIdx.x; t < BQ * chunks; t += blockDim.x) {
    uint32_t r = t / chunks, c = t - r * chunks;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (r < valid) v = __ldg(reinterpret_cast<const float4 *>(A + (r0 + r) * ld) + c);
    *reinterpret_cast<float4 *>(Rs + r * S + 4 * c) = v;
  }
}

// D[i][j] for rows of block blockIdx.x and columns [c0, c1).  A batched
// launch takes instance blockIdx.z's operands from the table; its blocks past
// the instance's rows or columns return.
template <int METRIC, int TQ, bool BATCH = false>
__global__ void __launch_bounds__(kTileThreads, 2)
    dense_kernel(const float *__restrict__ A, uint64_t na, const float *__restrict__ B, uint64_t nb,
                 uint32_t ld, uint32_t dp, float *__restrict__ D, uint64_t ldD, uint32_t cols_per_cta,
                 const DenseInst *__restrict__ tab = nullptr) {
  constexpr uint32_t BQ = 16 * TQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (BATCH) {
    const DenseInst &di = tab[blockIdx.z];
    A = di.A;
    na = di.na;
    B = di.B;
    nb = di.nb;
    D = di.D;
    ldD = di.ldD;
  }
  const uint32_t S = dp + 4;
  float *Rs = reinterpret_cast<float *>(smem_raw);
  float *Cs0 = Rs + BQ * S, *Cs1 = Cs0 + kTileCols * S;
  const int tq = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const uint64_t r0 = (uint64_t)blockIdx.x * BQ;
  if (r0 >= na) return;
  const uint32_t rvalid = (uint32_t)min((uint64_t)BQ, na - r0);
  const uint64_t c0 = (uint64_t)blockIdx.y * cols_per_cta;
  if (c0 >= nb) return;
  const uint64_t c1 = min(nb, c0 + cols_per_cta);
  stage_row_block<TQ>(Rs, S, A, ld, r0, rvalid, dp);
  const uint32_t ntiles = (uint32_t)((c1 - c0 + kTileCols - 1) / kTileCols);
  stage_rows_async(Cs0, S, B, ld, c0, (uint32_t)min((uint64_t)kTileCols, c1 - c0), dp);
  cp_async_commit();
  for (uint32_t t = 0; t < ntiles; t++) {
    float *cur = (t & 1) ? Cs1 : Cs0;
    float *nxt = (t & 1) ? Cs0 : Cs1;
    if (t + 1 < ntiles) {
      uint64_t b0 = c0 + (uint64_t)(t + 1) * kTileCols;
      stage_rows_async(nxt, S, B, ld, b0, (uint32_t)min((uint64_t)kTileCols, c1 - b0), dp);
    }
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    float acc[TQ][2];
    tile_distances<METRIC, TQ>(Rs, cur, S, dp, tq, tx, acc);
    const uint64_t cb = c0 + (uint64_t)t * kTileCols;
#pragma unroll
    for (int i = 0; i < TQ; i++) {
      uint32_t r = tq + 16 * i;
      if (r >= rvalid) continue;
#pragma unroll
      for (int j = 0; j < 2; j++) {
        uint64_t c = cb + tx + 16 * j;
        if (c < c1) D[(r0 + r) * ldD + c] = acc[i][j];
      }
    }
    __syncthreads();
  }
}

// best[i] = argmin_j (dist(A_i, B_j), j) over all nb rows of B.
template <int METRIC, int TQ>
__global__ void __launch_bounds__(kTileThreads, 2)
    argmin_kernel(const float *__restrict__ A, uint64_t na, const float *__restrict__ B, uint32_t nb,
                  uint32_t ld, uint32_t dp, uint32_t *__restrict__ best, float *__restrict__ bestd) {
  constexpr uint32_t BQ = 16 * TQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const uint32_t S = dp + 4;
  float *Rs = reinterpret_cast<float *>(smem_raw);
  float *Cs0 = Rs + BQ * S, *Cs1 = Cs0 + kTileCols * S;
  const int tq = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const uint64_t r0 = (uint64_t)blockIdx.x * BQ;
  const uint32_t rvalid = (uint32_t)min((uint64_t)BQ, na - r0);
  stage_row_block<TQ>(Rs, S, A, ld, r0, rvalid, dp);
  float bd[TQ];
  uint32_t bi[TQ];
#pragma unroll
  for (int i = 0; i < TQ; i++) {
    bd[i] = FLT_MAX;
    bi[i] = RBC_DUMMY;
  }
  const uint32_t ntiles = (nb + kTileCols - 1) / kTileCols;
  stage_rows_async(Cs0, S, B, ld, 0, min((uint32_t)kTileCols, nb), dp);
  cp_async_commit();
  for (uint32_t t = 0; t < ntiles; t++) {
    float *cur = (t & 1) ? Cs1 : Cs0;
    float *nxt = (t & 1) ? Cs0 : Cs1;
    if (t + 1 < ntiles) {
      uint32_t b0 = (t + 1) * kTileCols;
      stage_rows_async(nxt, S, B, ld, b0, min((uint32_t)kTileCols, nb - b0), dp);
    }
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    float acc[TQ][2];
    tile_distances<METRIC, TQ>(Rs, cur, S, dp, tq, tx, acc);
    const uint32_t cb = t * kTileCols;
#pragma unroll
    for (int i = 0; i < TQ; i++) {
#pragma unroll
      for (int j = 0; j < 2; j++) {
        uint32_t c = cb + tx + 16 * j;  // columns visited in increasing order per thread
        if (c < nb && acc[i][j] < bd[i]) {
          bd[i] = acc[i][j];
          bi[i] = c;
        }
      }
    }
    __syncthreads();
  }
  // reduce over the 16 threads sharing a row (one half warp)
#pragma unroll
  for (int i = 0; i < TQ; i++) {
    float d = bd[i];
    uint32_t id = bi[i];
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
      float od = __shfl_xor_sync(0xffffffffu, d, o);
      uint32_t oi = __shfl_xor_sync(0xffffffffu, id, o);
      if (pair_less(od, oi, d, id)) {
        d = od;
        id = oi;
      }
    }
    uint32_t r = tq + 16 * i;
    if (tx == 0 && r < rvalid) {
      best[r0 + r] = id;
      if (bestd) bestd[r0 + r] = d;
    }
  }
}

// counts[i] += #{j in chunk : dist(Q_i, X_j) < ranges[i]}; one CTA per 16*TQ
// queries (blockIdx.x) and chunk of `chunk` rows (blockIdx.y), so a small
// query set still fills the GPU.
template <int METRIC, int TQ>
__global__ void __launch_bounds__(kTileThreads, 2)
    range_count_kernel(const float *__restrict__ Q, uint64_t m, const float *__restrict__ X, uint64_t n,
                       uint32_t ld, uint32_t dp, const float *__restrict__ ranges,
                       uint32_t *__restrict__ counts, uint64_t chunk) {
  constexpr uint32_t BQ = 16 * TQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const uint32_t S = dp + 4;
  float *Rs = reinterpret_cast<float *>(smem_raw);
  float *Cs0 = Rs + BQ * S, *Cs1 = Cs0 + kTileCols * S;
  const int tq = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const uint64_t r0 = (uint64_t)blockIdx.x * BQ;
  const uint32_t rvalid = (uint32_t)min((uint64_t)BQ, m - r0);
  stage_row_block<TQ>(Rs, S, Q, ld, r0, rvalid, dp);
  float rg[TQ];
  uint32_t cnt[TQ];
#pragma unroll
  for (int i = 0; i < TQ; i++) {
    uint32_t r = tq + 16 * i;
    rg[i] = r < rvalid ? ranges[r0 + r] : 0.f;
    cnt[i] = 0;
  }
  const uint64_t c0 = (uint64_t)blockIdx.y * chunk, c1 = min(n, c0 + chunk);
  const uint64_t ntiles = (c1 - c0 + kTileCols - 1) / kTileCols;
  stage_rows_async(Cs0, S, X, ld, c0, (uint32_t)min((uint64_t)kTileCols, c1 - c0), dp);
  cp_async_commit();
  for (uint64_t t = 0; t < ntiles; t++) {
    float *cur = (t & 1) ? Cs1 : Cs0;
    float *nxt = (t & 1) ? Cs0 : Cs1;
    if (t + 1 < ntiles) {
      uint64_t b0 = c0 + (t + 1) * kTileCols;
      stage_rows_async(nxt, S, X, ld, b0, (uint32_t)min((uint64_t)kTileCols, c1 - b0), dp);
    }
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    float acc[TQ][2];
    tile_distances<METRIC, TQ>(Rs, cur, S, dp, tq, tx, acc);
    const uint64_t cb = c0 + t * kTileCols;
#pragma unroll
    for (int i = 0; i < TQ; i++)
#pragma unroll
      for (int j = 0; j < 2; j++) cnt[i] += (cb + tx + 16 * j < c1) && (acc[i][j] < rg[i]);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TQ; i++) {
    uint32_t c = cnt[i];
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    uint32_t r = tq + 16 * i;
    if (tx == 0 && r < rvalid && c) atomicAdd(counts + r0 + r, c);
  }
}

template <typename K>
cudaError_t prep(K kernel, size_t smem) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int METRIC, int TQ>
cudaError_t dense_tq(const float *A, uint64_t na, const float *B, uint64_t nb, uint32_t ld, uint32_t dp,
                     float *D, uint64_t ldD, cudaStream_t s) {
  size_t smem = rows_smem_bytes<TQ>(dp);
  cudaError_t e = prep(dense_kernel<METRIC, TQ>, smem);
  if (e != cudaSuccess) return e;
  const uint32_t cpc = 512;
  dim3 grid((unsigned)((na + 16 * TQ - 1) / (16 * TQ)), (unsigned)((nb + cpc - 1) / cpc));
  dense_kernel<METRIC, TQ><<<grid, kTileThreads, smem, s>>>(A, na, B, nb, ld, dp, D, ldD, cpc);
  return launched();
}

template <int METRIC, int TQ>
cudaError_t dense_batch_tq(const DenseInst *tab, uint32_t ninst, uint64_t na_max, uint64_t nb_max, uint32_t ld,
                           uint32_t dp, cudaStream_t s) {
  size_t smem = rows_smem_bytes<TQ>(dp);
  cudaError_t e = prep(dense_kernel<METRIC, TQ, true>, smem);
  if (e != cudaSuccess) return e;
  const uint32_t cpc = 512;
  dim3 grid((unsigned)((na_max + 16 * TQ - 1) / (16 * TQ)), (unsigned)((nb_max + cpc - 1) / cpc), ninst);
  dense_kernel<METRIC, TQ, true><<<grid, kTileThreads, smem, s>>>(nullptr, 0, nullptr, 0, ld, dp, nullptr, 0, cpc,
                                                                   tab);
  return launched();
}

template <int METRIC, int TQ>
cudaError_t argmin_tq(const float *A, uint64_t na, const float *B, uint32_t nb, uint32_t ld, uint32_t dp,
                      uint32_t *best, float *bestd, cudaStream_t s) {
  size_t smem = rows_smem_bytes<TQ>(dp);
  cudaError_t e = prep(argmin_kernel<METRIC, TQ>, smem);
  if (e != cudaSuccess) return e;
  unsigned grid = (unsigned)((na + 16 * TQ - 1) / (16 * TQ));
  argmin_kernel<METRIC, TQ><<<grid, kTileThreads, smem, s>>>(A, na, B, nb, ld, dp, best, bestd);
  return launched();
}

template <int METRIC, int TQ>
cudaError_t range_tq(const float *Q, uint64_t m, const float *X, uint64_t n, uint32_t ld, uint32_t dp,
                     const float *ranges, uint32_t *counts, cudaStream_t s) {
  size_t smem = rows_smem_bytes<TQ>(dp);
  cudaError_t e = prep(range_count_kernel<METRIC, TQ>, smem);
  if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, m * sizeof(uint32_t), s);
  if (e != cudaSuccess || n == 0) return e;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // row chunks so that query tiles x chunks covers the SMs about four times over
  const uint64_t qtiles = (m + 16 * TQ - 1) / (16 * TQ);
  uint64_t nchunks = std::min<uint64_t>((4ull * sms + qtiles - 1) / qtiles, (n + 1023) / 1024);
  nchunks = std::max<uint64_t>(1, std::min<uint64_t>(nchunks, 65535));
  const uint64_t chunk = ((n + nchunks - 1) / nchunks + kTileCols - 1) / kTileCols * kTileCols;
  nchunks = (n + chunk - 1) / chunk;
  for (uint64_t q0 = 0; q0 < qtiles; q0 += 1u << 30) {  // grid.x limit
    const uint64_t nt = std::min<uint64_t>(qtiles - q0, 1u << 30);
    range_count_kernel<METRIC, TQ><<<dim3((unsigned)nt, (unsigned)nchunks), kTileThreads, smem, s>>>(
        Q + q0 * 16 * TQ * ld, m - q0 * 16 * TQ, X, n, ld, dp, ranges + q0 * 16 * TQ, counts + q0 * 16 * TQ, chunk);
    if ((e = launched()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

#define RBC_DISPATCH(metric, dp, FN, ...)                                               \
  do {                                                                                  \
    int tqv_ = search_tq_for(dp);                                                       \
    if ((metric) == RBC_L1)                                                             \
      return tqv_ == 4 ? FN<RBC_L1, 4>(__VA_ARGS__)                                     \
                       : tqv_ == 2 ? FN<RBC_L1, 2>(__VA_ARGS__) : FN<RBC_L1, 1>(__VA_ARGS__); \
    return tqv_ == 4 ? FN<RBC_L2, 4>(__VA_ARGS__)                                       \
                     : tqv_ == 2 ? FN<RBC_L2, 2>(__VA_ARGS__) : FN<RBC_L2, 1>(__VA_ARGS__);   \
  } while (0)

}  // namespace

cudaError_t launch_dense_dist(int metric, const float *A, uint64_t na, const float *B, uint64_t nb,
                              uint32_t ld, uint32_t dp, float *D, uint64_t ldD, cudaStream_t s) {
  if (na == 0 || nb == 0) return cudaSuccess;
  RBC_DISPATCH(metric, dp, dense_tq, A, na, B, nb, ld, dp, D, ldD, s);
}

cudaError_t launch_dense_dist_batch(int metric, const DenseInst *tab, uint32_t ninst, uint64_t na_max,
                                    uint64_t nb_max, uint32_t ld, uint32_t dp, cudaStream_t s) {
  if (ninst == 0 || na_max == 0 || nb_max == 0) return cudaSuccess;
  RBC_DISPATCH(metric, dp, dense_batch_tq, tab, ninst, na_max, nb_max, ld, dp, s);
}

cudaError_t launch_argmin(int metric, const float *A, uint64_t na, const float *B, uint32_t nb,
                          uint32_t ld, uint32_t dp, uint32_t *best, float *bestd, cudaStream_t s) {
  if (na == 0) return cudaSuccess;
  RBC_DISPATCH(metric, dp, argmin_tq, A, na, B, nb, ld, dp, best, bestd, s);
}

cudaError_t launch_range_count(int metric, const float *Q, uint64_t m, const float *X, uint64_t n,
                               uint32_t ld, uint32_t dp, const float *ranges, uint32_t *counts,
                               cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  RBC_DISPATCH(metric, dp, range_tq, Q, m, X, n, ld, dp, ranges, counts, s);
}

}  // namespace rbc
