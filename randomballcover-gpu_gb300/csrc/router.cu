// router.cu -- the learned list router: a small MLP trained on the GPU with
// hand-written forward, backward and optimiser kernels.
//
// Model: d -> H -> H -> L (L = number of lists), GELU after the two hidden
// layers, logits out.  Master weights are FP32; the forward and backward
// passes read a BF16 copy of the weights (refreshed after every update) and
// accumulate in FP32.  Training minimises softmax cross-entropy against the
// list that owns each training query's exact nearest neighbour -- a label the
// RBC itself produces (rbc_owner_labels) -- with Adam.  At query time the
// router's top-P lists are searched first, so the k-th distance is tight
// before the pruning round; exact pruning still decides every other list, so
// results stay exact whatever the router predicts.
//
// Kernels:
//   gemm_kernel      C = op(A) op(B) (+ bias), 64x64 tiles, 4x4 per thread,
//                    FP32 or BF16 operands staged as FP32 in shared memory
//   bias_gelu        h = x + b, a = GELU(h) (exact erf form), h kept
//   gelu_backward    dh = da * GELU'(h)
//   softmax_xent     per row: loss and dz = (softmax(z) - onehot(y)) / B
//   tau_loss         distance head: loss (z - t)^2 and dz = 2 (z - t) / B
//                    (rows without a target add nothing)
//   colsum           bias gradients
//   adam             m, v, w updates and the BF16 weight copy
#include <cuda_bf16.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.cuh"
#include "rbc_common.cuh"
#include "router.cuh"

namespace rbc {

namespace {

constexpr int kGT = 64, kGK = 16;  // GEMM tile (M, N) and K step

template <typename T>
__device__ __forceinline__ float ldf(const T *p) {
  return static_cast<float>(*p);
}
template <>
__device__ __forceinline__ float ldf<__nv_bfloat16>(const __nv_bfloat16 *p) {
  return __bfloat162float(*p);
}

// C[m][n] = sum_k A(m,k) B(k,n) + bias[n];  A(m,k) = TA ? A[k lda + m] : A[m lda + k],
// B(k,n) = TB ? B[n ldb + k] : B[k ldb + n].  accumulate: C += instead of =.
template <bool TA, bool TB, typename AT, typename BT>
__global__ void __launch_bounds__(256) gemm_kernel(const AT *__restrict__ A, uint32_t lda, const BT *__restrict__ B,
                                                   uint32_t ldb, float *__restrict__ C, uint32_t ldc, uint32_t M,
                                                   uint32_t N, uint32_t K, const float *__restrict__ bias,
                                                   int accumulate) {
  __shared__ float As[kGK][kGT + 4];
  __shared__ float Bs[kGK][kGT + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const uint32_t m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  float acc[4][4] = {};
  for (uint32_t k0 = 0; k0 < K; k0 += kGK) {
    for (int t = threadIdx.x; t < kGK * kGT; t += 256) {
      int kk, mm;
      if (TA) {
        kk = t / kGT;
        mm = t % kGT;
      } else {
        mm = t / kGK;
        kk = t % kGK;
      }
      const uint32_t gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < K) v = TA ? ldf(A + (uint64_t)gk * lda + gm) : ldf(A + (uint64_t)gm * lda + gk);
      As[kk][mm] = v;
    }
    for (int t = threadIdx.x; t < kGK * kGT; t += 256) {
      int kk, nn;
      if (TB) {
        nn = t / kGK;
        kk = t % kGK;
      } else {
        kk = t / kGT;
        nn = t % kGT;
      }
      const uint32_t gn = n0 + nn, gk = k0 + kk;
      float v = 0.f;
      if (gn < N && gk < K) v = TB ? ldf(B + (uint64_t)gn * ldb + gk) : ldf(B + (uint64_t)gk * ldb + gn);
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const uint32_t gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const uint32_t gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      float v = acc[i][j] + (bias ? bias[gn] : 0.f);
      float *c = C + (uint64_t)gm * ldc + gn;
      *c = accumulate ? *c + v : v;
    }
  }
}

template <bool TA, bool TB, typename AT, typename BT>
cudaError_t gemm(const AT *A, uint32_t lda, const BT *B, uint32_t ldb, float *C, uint32_t ldc, uint32_t M, uint32_t N,
                 uint32_t K, const float *bias, bool accumulate, cudaStream_t s) {
  dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT);
  gemm_kernel<TA, TB, AT, BT><<<grid, 256, 0, s>>>(A, lda, B, ldb, C, ldc, M, N, K, bias, accumulate ? 1 : 0);
  return launched();
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
  const float pdf = 0.3989422804014327f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// a = GELU(h), in place on h's copy: h stays the pre-activation.
__global__ void gelu_kernel(const float *__restrict__ h, float *__restrict__ a, uint64_t total) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < total) a[i] = gelu(h[i]);
}

__global__ void gelu_backward_kernel(const float *__restrict__ h, float *__restrict__ g, uint64_t total) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < total) g[i] *= gelu_grad(h[i]);
}

// One block per row: loss_i = logsumexp(z) - z_y; dz = (softmax(z) - onehot(y)) * scale.
__global__ void softmax_xent_kernel(float *__restrict__ z, uint32_t L, const uint32_t *__restrict__ y,
                                    float *__restrict__ loss, float scale, int want_grad) {
  __shared__ float red[32];
  const uint64_t r = blockIdx.x;
  float *row = z + r * L;
  float mx = -INFINITY;
  for (uint32_t j = threadIdx.x; j < L; j += blockDim.x) mx = fmaxf(mx, row[j]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  mx = -INFINITY;
  for (uint32_t w = 0; w < blockDim.x / 32; w++) mx = fmaxf(mx, red[w]);
  __syncthreads();
  float se = 0.f;
  for (uint32_t j = threadIdx.x; j < L; j += blockDim.x) se += expf(row[j] - mx);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) se += __shfl_xor_sync(0xffffffffu, se, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = se;
  __syncthreads();
  se = 0.f;
  for (uint32_t w = 0; w < blockDim.x / 32; w++) se += red[w];
  const float lse = mx + logf(se);
  const uint32_t yl = y[r];
  if (threadIdx.x == 0 && loss) loss[r] = lse - row[yl];
  __syncthreads();
  if (!want_grad) return;
  for (uint32_t j = threadIdx.x; j < L; j += blockDim.x) {
    float p = expf(row[j] - lse);
    row[j] = (p - (j == yl ? 1.f : 0.f)) * scale;
  }
}

// The distance head's squared error on the batch's normalised targets (NaN:
// no target); zt becomes its gradient.
__global__ void tau_loss_kernel(float *__restrict__ zt, const float *__restrict__ yt, uint32_t b,
                                float *__restrict__ loss, float scale) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= b) return;
  const float t = yt[r];
  const float e = isfinite(t) ? zt[r] - t : 0.f;
  if (loss) loss[r] += e * e;
  zt[r] = 2.f * e * scale;
}

__global__ void tau_from_head_kernel(const float *__restrict__ z, const float *__restrict__ near, uint64_t m, float mu,
                                     float sigma, float margin, float *__restrict__ tau) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  const float v = near[i] * __expf(fmaf(sigma, z[i] + margin, mu));
  tau[i] = isfinite(v) ? fminf(v * 1.0001f, FLT_MAX) : FLT_MAX;
}

// out[n] = sum over rows of g[r][n] (bias gradients).
__global__ void colsum_kernel(const float *__restrict__ g, uint32_t rows, uint32_t N, float *__restrict__ out) {
  uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (uint32_t r = 0; r < rows; r++) s += g[(uint64_t)r * N + n];
  out[n] = s;
}

__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m1,
                            float *__restrict__ m2, __nv_bfloat16 *__restrict__ wb, uint64_t total, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= total) return;
  float gi = g[i];
  float a = b1 * m1[i] + (1.f - b1) * gi;
  float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  float wi = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
  w[i] = wi;
  wb[i] = __float2bfloat16_rn(wi);
}

__global__ void to_bf16_flat(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb, uint64_t total) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < total) wb[i] = __float2bfloat16_rn(w[i]);
}

// Deterministic initialisation: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) from a counter hash.
__global__ void init_kernel(float *__restrict__ w, uint64_t total, uint64_t seed, uint64_t offset, float scale) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= total) return;
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + offset + i;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  float u = (float)(z >> 40) * 5.9604644775390625e-08f;
  w[i] = (2.f * u - 1.f) * scale;
}

// Gather rows of the training set for a batch (order[] holds row indices),
// with their labels and (distance head) targets.
__global__ void gather_batch_kernel(const float *__restrict__ Q, uint32_t ldq, uint32_t d,
                                    const uint32_t *__restrict__ order, const uint32_t *__restrict__ labels,
                                    const float *__restrict__ tsrc, uint32_t batch, float *__restrict__ X,
                                    uint32_t *__restrict__ y, float *__restrict__ yt) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= (uint64_t)batch * d) return;
  uint32_t r = (uint32_t)(i / d), c = (uint32_t)(i - (uint64_t)r * d);
  uint32_t src = order[r];
  X[i] = Q[(uint64_t)src * ldq + c];
  if (c == 0) {
    y[r] = labels[src];
    if (yt) yt[r] = tsrc ? tsrc[src] : __int_as_float(0x7fc00000);
  }
}

unsigned blocks(uint64_t total, unsigned t = 256) { return (unsigned)((total + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------------ host
size_t Router::nparams() const {
  return (size_t)H * d + H + (size_t)H * H + H + (size_t)(L + T) * H + (L + T);
}

cudaError_t Router::alloc_batch(uint32_t b, cudaStream_t s) {
  if (b <= cap) return cudaSuccess;
  for (void *p : {(void *)X, (void *)y, (void *)h1, (void *)a1, (void *)h2, (void *)a2, (void *)z, (void *)ga,
                  (void *)gb, (void *)loss, (void *)yt, (void *)zt})
    if (p) cudaFreeAsync(p, s);
  yt = zt = nullptr;
  cudaError_t e = cudaSuccess;
  auto al = [&](auto **p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMallocAsync((void **)p, bytes, s);
  };
  al(&X, (size_t)b * d * 4);
  al(&y, (size_t)b * 4);
  al(&h1, (size_t)b * H * 4);
  al(&a1, (size_t)b * H * 4);
  al(&h2, (size_t)b * H * 4);
  al(&a2, (size_t)b * H * 4);
  al(&z, (size_t)b * L * 4);
  al(&ga, (size_t)b * H * 4);
  al(&gb, (size_t)b * H * 4);
  al(&loss, (size_t)b * 4);
  if (T) {
    al(&yt, (size_t)b * 4);
    al(&zt, (size_t)b * 4);
  }
  cap = e == cudaSuccess ? b : 0;
  return e;
}

// Forward pass of `b` rows of X (b x d, stride d) into logits z (b x L) and,
// with the distance head, its outputs zt_out (b); either output may be null.
cudaError_t Router::forward(const float *Xin, uint32_t ldx, uint32_t b, float *zout, cudaStream_t s, float *zt_out) {
  const __nv_bfloat16 *W1 = wb, *W2 = wb + (size_t)H * d + H, *W3 = W2 + (size_t)H * H + H;
  const float *b1 = w + (size_t)H * d, *b2 = b1 + H + (size_t)H * H, *b3 = b2 + H + (size_t)(L + T) * H;
  cudaError_t e = gemm<false, true>(Xin, ldx, W1, d, h1, H, b, H, d, b1, false, s);
  if (e == cudaSuccess) {
    gelu_kernel<<<blocks((uint64_t)b * H), 256, 0, s>>>(h1, a1, (uint64_t)b * H);
    e = launched();
  }
  if (e == cudaSuccess) e = gemm<false, true>(a1, H, W2, H, h2, H, b, H, H, b2, false, s);
  if (e == cudaSuccess) {
    gelu_kernel<<<blocks((uint64_t)b * H), 256, 0, s>>>(h2, a2, (uint64_t)b * H);
    e = launched();
  }
  if (e == cudaSuccess && zout) e = gemm<false, true>(a2, H, W3, H, zout, L, b, L, H, b3, false, s);
  if (e == cudaSuccess && T && zt_out)
    e = gemm<false, true>(a2, H, W3 + (size_t)L * H, H, zt_out, 1, b, 1, H, b3 + L, false, s);
  return e;
}

// Loss and gradients (into g) of the batch already in X / y; z is overwritten by dz.
cudaError_t Router::forward_backward(uint32_t b, cudaStream_t s) {
  const __nv_bfloat16 *W2 = wb + (size_t)H * d + H, *W3 = W2 + (size_t)H * H + H;
  float *gW1 = g, *gb1 = g + (size_t)H * d, *gW2 = gb1 + H, *gb2 = gW2 + (size_t)H * H, *gW3 = gb2 + H,
        *gb3 = gW3 + (size_t)(L + T) * H;
  cudaError_t e = forward(X, d, b, z, s, zt);
  if (e != cudaSuccess) return e;
  softmax_xent_kernel<<<b, 256, 0, s>>>(z, L, y, loss, 1.f / b, 1);
  if ((e = launched()) != cudaSuccess) return e;
  if (T) {
    tau_loss_kernel<<<blocks(b), 256, 0, s>>>(zt, yt, b, loss, 1.f / b);
    if ((e = launched()) != cudaSuccess) return e;
  }
  // layer 3: dW3 = dz^T a2, db3 = colsum dz, da2 = dz W3 (each with the
  // distance head's row when there is one)
  if ((e = gemm<true, false>(z, L, a2, H, gW3, H, L, H, b, nullptr, false, s)) != cudaSuccess) return e;
  colsum_kernel<<<blocks(L), 256, 0, s>>>(z, b, L, gb3);
  if ((e = launched()) != cudaSuccess) return e;
  if ((e = gemm<false, false>(z, L, W3, H, ga, H, b, H, L, nullptr, false, s)) != cudaSuccess) return e;
  if (T) {
    if ((e = gemm<true, false>(zt, 1, a2, H, gW3 + (size_t)L * H, H, 1, H, b, nullptr, false, s)) != cudaSuccess)
      return e;
    colsum_kernel<<<1, 32, 0, s>>>(zt, b, 1, gb3 + L);
    if ((e = launched()) != cudaSuccess) return e;
    if ((e = gemm<false, false>(zt, 1, W3 + (size_t)L * H, H, ga, H, b, H, 1, nullptr, true, s)) != cudaSuccess)
      return e;
  }
  gelu_backward_kernel<<<blocks((uint64_t)b * H), 256, 0, s>>>(h2, ga, (uint64_t)b * H);
  if ((e = launched()) != cudaSuccess) return e;
  // layer 2
  if ((e = gemm<true, false>(ga, H, a1, H, gW2, H, H, H, b, nullptr, false, s)) != cudaSuccess) return e;
  colsum_kernel<<<blocks(H), 256, 0, s>>>(ga, b, H, gb2);
  if ((e = launched()) != cudaSuccess) return e;
  if ((e = gemm<false, false>(ga, H, W2, H, gb, H, b, H, H, nullptr, false, s)) != cudaSuccess) return e;
  gelu_backward_kernel<<<blocks((uint64_t)b * H), 256, 0, s>>>(h1, gb, (uint64_t)b * H);
  if ((e = launched()) != cudaSuccess) return e;
  // layer 1
  if ((e = gemm<true, false>(gb, H, X, d, gW1, d, H, d, b, nullptr, false, s)) != cudaSuccess) return e;
  colsum_kernel<<<blocks(H), 256, 0, s>>>(gb, b, H, gb1);
  return launched();
}

cudaError_t Router::adam_step(float lr, cudaStream_t s) {
  step++;
  version++;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  const uint64_t P = nparams();
  adam_kernel<<<blocks(P), 256, 0, s>>>(w, g, m1, m2, wb, P, lr, b1, b2, eps, c1, c2);
  return launched();
}

cudaError_t Router::refresh_bf16(cudaStream_t s) {
  version++;
  const uint64_t P = nparams();
  to_bf16_flat<<<blocks(P), 256, 0, s>>>(w, wb, P);
  return launched();
}

cudaError_t Router::init(uint64_t seed, cudaStream_t s) {
  const uint64_t sizes[6] = {(uint64_t)H * d, H, (uint64_t)H * H, H, (uint64_t)(L + T) * H, L + T};
  const float fan[6] = {(float)d, (float)d, (float)H, (float)H, (float)H, (float)H};
  uint64_t off = 0;
  for (int i = 0; i < 6; i++) {
    init_kernel<<<blocks(sizes[i]), 256, 0, s>>>(w + off, sizes[i], seed, off, 1.f / sqrtf(fan[i]));
    cudaError_t e = launched();
    if (e != cudaSuccess) return e;
    off += sizes[i];
  }
  cudaError_t e = cudaMemsetAsync(m1, 0, nparams() * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(m2, 0, nparams() * 4, s);
  step = 0;
  return e == cudaSuccess ? refresh_bf16(s) : e;
}

cudaError_t Router::gather(const float *Q, uint32_t ldq, const uint32_t *order, const uint32_t *labels, uint32_t b,
                           cudaStream_t s) {
  gather_batch_kernel<<<blocks((uint64_t)b * d), 256, 0, s>>>(Q, ldq, d, order, labels, tau_src, b, X, y,
                                                              T ? yt : nullptr);
  return launched();
}

// The distance head's outputs (normalised units) for b rows, on the queries'
// inference path: tensor-core layers when hidden allows, else the training
// forward.
cudaError_t Router::head_outputs(const float *Xin, uint64_t ldx, uint64_t b, float *zt_out, uint32_t *err,
                                 cudaStream_t s) {
  if (!T) return cudaErrorInvalidValue;
  const uint32_t chunk = tc_ok() ? (1u << 18) : 4096;
  cudaError_t e = tc_ok() ? cudaSuccess : alloc_batch(chunk, s);
  for (uint64_t i = 0; i < b && e == cudaSuccess; i += chunk) {
    const uint32_t cb = (uint32_t)std::min<uint64_t>(chunk, b - i);
    e = tc_ok() ? forward_tc_head(Xin + i * ldx, (uint32_t)ldx, cb, zt_out + i, err, s)
                : forward(Xin + i * ldx, (uint32_t)ldx, cb, nullptr, s, zt_out + i);
  }
  return e;
}

// Predicted k-th distances: tau = near exp(mu + sigma (z + margin)), near the
// distance to the query's nearest representative.
cudaError_t Router::predict_tau(const float *Xin, uint32_t ldx, uint32_t b, const float *near, float *tau,
                                uint32_t *err, cudaStream_t s) {
  cudaError_t e = head_outputs(Xin, ldx, b, tau, err, s);
  if (e == cudaSuccess) e = launch_tau_from_head(tau, near, b, tau_mu, tau_sigma, tau_margin, tau, s);
  return e;
}

Router::~Router() {
  for (void *p : {(void *)w, (void *)g, (void *)m1, (void *)m2, (void *)wb, (void *)X, (void *)y, (void *)h1,
                  (void *)a1, (void *)h2, (void *)a2, (void *)z, (void *)ga, (void *)gb, (void *)loss, (void *)xb,
                  (void *)h1b, (void *)h2b, (void *)w1p, (void *)yt, (void *)zt})
    if (p) cudaFree(p);
}

namespace {

// One warp per row: columns [0, Pn) of the probe table take the Pn nearest
// representatives (table `nearest`, Pn wide), columns [Pn, Pn + P) the P
// largest logits (ties to the lower list index) that are not among them.
__global__ void router_probes_kernel(const float *__restrict__ z, uint64_t m, uint32_t L, uint32_t P, uint32_t Pn,
                                     const uint32_t *__restrict__ nearest, const float *__restrict__ nearest_d,
                                     uint32_t *__restrict__ probe, float *__restrict__ probed) {
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (q >= m) return;
  const float *row = z + q * L;
  const uint32_t W = Pn + P;
  uint32_t taken[16];
  for (uint32_t p = 0; p < Pn; p++) {
    taken[p] = nearest[q * Pn + p];
    if (lane == 0) {
      probe[q * W + p] = taken[p];
      probed[q * W + p] = nearest_d[q * Pn + p];
    }
  }
  for (uint32_t p = 0; p < P; p++) {
    float bv = -INFINITY;
    uint32_t bi = RBC_DUMMY;
    for (uint32_t j = lane; j < L; j += 32) {
      bool used = false;
      for (uint32_t t = 0; t < Pn + p; t++) used |= taken[t] == j;
      float v = row[j];
      if (!used && (v > bv || (v == bv && j < bi))) {
        bv = v;
        bi = j;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    taken[Pn + p] = bi;
    if (lane == 0) {
      probe[q * W + Pn + p] = bi;
      probed[q * W + Pn + p] = 0.f;
    }
  }
}

__global__ void owner_lookup_kernel(const uint32_t *__restrict__ ids, uint64_t m, uint32_t ldo,
                                    const uint32_t *__restrict__ owner, uint32_t *__restrict__ labels) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < m) {
    uint32_t id = ids[i * ldo];
    labels[i] = id == RBC_DUMMY ? 0u : owner[id];
  }
}

}  // namespace

cudaError_t launch_router_probes(const float *logits, uint64_t m, uint32_t L, uint32_t P, uint32_t Pn,
                                 const uint32_t *nearest, const float *nearest_d, uint32_t *probe, float *probed,
                                 cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  if (Pn + P > 16) return cudaErrorInvalidValue;
  router_probes_kernel<<<blocks(m * 32), 256, 0, s>>>(logits, m, L, P, Pn, nearest, nearest_d, probe, probed);
  return launched();
}

cudaError_t launch_tau_from_head(const float *z, const float *near, uint64_t m, float mu, float sigma, float margin,
                                 float *tau, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  tau_from_head_kernel<<<blocks(m), 256, 0, s>>>(z, near, m, mu, sigma, margin, tau);
  return launched();
}

cudaError_t launch_owner_lookup(const uint32_t *ids, uint64_t m, uint32_t ldo, const uint32_t *owner,
                                uint32_t *labels, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  owner_lookup_kernel<<<blocks(m), 256, 0, s>>>(ids, m, ldo, owner, labels);
  return launched();
}

}  // namespace rbc

// ====================================================================== C ABI
using namespace rbc;

#define RCK(expr)                                       \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #expr); \
  } while (0)

extern "C" {

namespace {

int create_router(uint32_t d, uint32_t hidden, uint32_t num_lists, uint32_t heads, uint64_t seed, rbc_router **out) {
  if (!out) return fail(RBC_ERR_INVALID, "rbc_router_create: out is NULL");
  *out = nullptr;
  if (d == 0 || hidden == 0 || num_lists == 0) return fail(RBC_ERR_INVALID, "rbc_router_create: zero size");
  rbc_router *rt = new rbc_router();
  Router &r = rt->r;
  r.d = d;
  r.H = hidden;
  r.L = num_lists;
  r.T = heads;
  const size_t P = r.nparams();
  cudaError_t e = cudaMalloc(&r.w, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&r.g, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&r.m1, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&r.m2, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&r.wb, P * 2);
  if (e == cudaSuccess) e = r.init(seed, nullptr);
  if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
  if (e != cudaSuccess) {
    delete rt;
    return cuda_fail(e, "rbc_router_create");
  }
  *out = rt;
  return RBC_OK;
}

// Epochs of Adam over rows [0, n) in shuffled batches; the loss of the last
// batch (mean over its rows) goes to final_loss.
int train_loop(Router &r, const float *dQ, uint64_t n, uint32_t ldq, const uint32_t *dLabels, uint32_t epochs,
               uint32_t batch, float lr, uint64_t seed, float *final_loss, cudaStream_t s) {
  const uint32_t b = (uint32_t)std::min<uint64_t>(batch, n);
  RCK(r.alloc_batch(b, s));
  std::vector<uint32_t> order(n);
  uint32_t *dorder = nullptr;
  RCK(cudaMallocAsync(&dorder, n * 4, s));
  uint64_t state = seed * 0x9E3779B97F4A7C15ull + 1;
  auto next = [&]() {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  for (uint32_t ep = 0; ep < epochs; ep++) {
    for (uint64_t i = 0; i < n; i++) order[i] = (uint32_t)i;
    for (uint64_t i = n - 1; i > 0; i--) std::swap(order[i], order[next() % (i + 1)]);
    RCK(cudaMemcpyAsync(dorder, order.data(), n * 4, cudaMemcpyHostToDevice, s));
    RCK(cudaStreamSynchronize(s));  // order[] is reshuffled next epoch
    const uint64_t steps = n / b;
    for (uint64_t t = 0; t < steps; t++) {
      RCK(r.gather(dQ, ldq, dorder + t * b, dLabels, b, s));
      RCK(r.forward_backward(b, s));
      RCK(r.adam_step(lr, s));
    }
  }
  if (final_loss) {
    std::vector<float> l(b);
    RCK(cudaMemcpyAsync(l.data(), r.loss, b * 4, cudaMemcpyDeviceToHost, s));
    RCK(cudaStreamSynchronize(s));
    double last = 0;
    for (float v : l) last += v;
    *final_loss = (float)(last / b);
  }
  RCK(cudaFreeAsync(dorder, s));
  RCK(cudaStreamSynchronize(s));
  return RBC_OK;
}

}  // namespace

int rbc_router_create(uint32_t d, uint32_t hidden, uint32_t num_lists, uint64_t seed, rbc_router **out) {
  return create_router(d, hidden, num_lists, 0, seed, out);
}

int rbc_router_create_with_distance(uint32_t d, uint32_t hidden, uint32_t num_lists, uint64_t seed,
                                    rbc_router **out) {
  return create_router(d, hidden, num_lists, 1, seed, out);
}

int rbc_router_destroy(rbc_router *router) {
  delete router;
  return RBC_OK;
}

int rbc_router_num_params(const rbc_router *router, uint64_t *count) {
  if (!router || !count) return fail(RBC_ERR_INVALID, "rbc_router_num_params: NULL argument");
  *count = router->r.nparams();
  return RBC_OK;
}

int rbc_router_get_params(const rbc_router *router, float *h_params) {
  if (!router || !h_params) return fail(RBC_ERR_INVALID, "rbc_router_get_params: NULL argument");
  RCK(cudaMemcpy(h_params, router->r.w, router->r.nparams() * 4, cudaMemcpyDeviceToHost));
  return RBC_OK;
}

int rbc_router_set_params(rbc_router *router, const float *h_params) {
  if (!router || !h_params) return fail(RBC_ERR_INVALID, "rbc_router_set_params: NULL argument");
  RCK(cudaMemcpy(router->r.w, h_params, router->r.nparams() * 4, cudaMemcpyHostToDevice));
  RCK(router->r.refresh_bf16(nullptr));
  RCK(cudaStreamSynchronize(nullptr));
  return RBC_OK;
}

int rbc_router_gradients(rbc_router *router, const float *dQ, uint32_t batch, uint32_t ldq, const uint32_t *dLabels,
                         float *loss, float *h_grads, void *stream) {
  if (!router || !dQ || !dLabels || batch == 0) return fail(RBC_ERR_INVALID, "rbc_router_gradients: bad argument");
  if (ldq < router->r.d) return fail(RBC_ERR_INVALID, "rbc_router_gradients: ldq < d");
  Router &r = router->r;
  cudaStream_t s = (cudaStream_t)stream;
  RCK(r.alloc_batch(batch, s));
  std::vector<uint32_t> order(batch);
  for (uint32_t i = 0; i < batch; i++) order[i] = i;
  uint32_t *dorder = nullptr;
  RCK(cudaMallocAsync(&dorder, batch * 4, s));
  RCK(cudaMemcpyAsync(dorder, order.data(), batch * 4, cudaMemcpyHostToDevice, s));
  RCK(r.gather(dQ, ldq, dorder, dLabels, batch, s));
  RCK(r.forward_backward(batch, s));
  std::vector<float> l(batch);
  RCK(cudaMemcpyAsync(l.data(), r.loss, batch * 4, cudaMemcpyDeviceToHost, s));
  if (h_grads) RCK(cudaMemcpyAsync(h_grads, r.g, r.nparams() * 4, cudaMemcpyDeviceToHost, s));
  RCK(cudaFreeAsync(dorder, s));
  RCK(cudaStreamSynchronize(s));
  if (loss) {
    double t = 0;
    for (float v : l) t += v;
    *loss = (float)(t / batch);
  }
  return RBC_OK;
}

int rbc_router_train(rbc_router *router, const float *dQ, uint64_t n, uint32_t ldq, const uint32_t *dLabels,
                     uint32_t epochs, uint32_t batch, float lr, uint64_t seed, float *final_loss, void *stream) {
  if (!router || !dQ || !dLabels || n == 0 || batch == 0) return fail(RBC_ERR_INVALID, "rbc_router_train: bad argument");
  if (ldq < router->r.d) return fail(RBC_ERR_INVALID, "rbc_router_train: ldq < d");
  if (n >= 0xFFFFFFFFull) return fail(RBC_ERR_INVALID, "rbc_router_train: too many samples");
  Router &r = router->r;
  r.tau_src = nullptr;  // a distance head, if any, gets no targets here
  return train_loop(r, dQ, n, ldq, dLabels, epochs, batch, lr, seed, final_loss, (cudaStream_t)stream);
}

int rbc_router_train_with_distance(rbc_router *router, const float *dQ, uint64_t n, uint32_t ldq,
                                   const uint32_t *dLabels, const float *dDist, const float *dNear, uint32_t epochs,
                                   uint32_t batch, float lr, uint64_t seed, float *final_loss, void *stream) {
  if (!router || !dQ || !dLabels || !dDist || !dNear || n == 0 || batch == 0)
    return fail(RBC_ERR_INVALID, "rbc_router_train_with_distance: bad argument");
  Router &r = router->r;
  if (!r.T) return fail(RBC_ERR_INVALID, "rbc_router_train_with_distance: the router has no distance head");
  if (ldq < r.d) return fail(RBC_ERR_INVALID, "rbc_router_train_with_distance: ldq < d");
  if (n >= 0xFFFFFFFFull) return fail(RBC_ERR_INVALID, "rbc_router_train_with_distance: too many samples");
  cudaStream_t s = (cudaStream_t)stream;
  // targets: log of each k-th distance over the nearest representative's,
  // normalised by the mean and spread of the usable ones (both distances
  // finite and positive; the others train the lists only)
  std::vector<float> h(n), hn(n);
  RCK(cudaMemcpyAsync(h.data(), dDist, n * 4, cudaMemcpyDeviceToHost, s));
  RCK(cudaMemcpyAsync(hn.data(), dNear, n * 4, cudaMemcpyDeviceToHost, s));
  RCK(cudaStreamSynchronize(s));
  auto usable = [](float v) { return std::isfinite(v) && v > 0.f && v < FLT_MAX; };
  double sum = 0, sum2 = 0;
  uint64_t cnt = 0;
  for (uint64_t i = 0; i < n; i++) {
    if (usable(h[i]) && usable(hn[i])) {
      const double l = std::log((double)h[i] / (double)hn[i]);
      h[i] = (float)l;
      sum += l;
      sum2 += l * l;
      cnt++;
    } else {
      h[i] = NAN;
    }
  }
  if (cnt == 0) return fail(RBC_ERR_INVALID, "rbc_router_train_with_distance: no finite positive distance");
  const double mu = sum / cnt, var = std::max(sum2 / cnt - mu * mu, 1e-12);
  r.tau_mu = (float)mu;
  r.tau_sigma = (float)std::sqrt(var);
  for (uint64_t i = 0; i < n; i++)
    if (std::isfinite(h[i])) h[i] = (float)((h[i] - mu) / r.tau_sigma);
  float *dt = nullptr;
  RCK(cudaMallocAsync(&dt, n * 4, s));
  RCK(cudaMemcpyAsync(dt, h.data(), n * 4, cudaMemcpyHostToDevice, s));
  // the last 2 % of the rows are held out to calibrate the margin (all rows
  // serve both when there are too few)
  const uint64_t hold = n >= 1000 ? n / 50 : 0, ntrain = n - hold;
  r.tau_src = dt;
  int rc = train_loop(r, dQ, ntrain, ldq, dLabels, epochs, batch, lr, seed, final_loss, s);
  r.tau_src = nullptr;
  if (rc == RBC_OK) {
    // margin: the 99.5th percentile of (target - prediction) over the held-out
    // rows, predicted on the queries' own inference path
    const uint64_t c0 = hold ? ntrain : 0, nc = hold ? hold : n;
    float *z = nullptr;
    uint32_t *err = nullptr, herr = 0;
    RCK(cudaMallocAsync(&z, nc * 4, s));
    RCK(cudaMallocAsync(&err, 4, s));
    RCK(cudaMemsetAsync(err, 0, 4, s));
    const float keep = r.tau_margin;
    cudaError_t e = r.head_outputs(dQ + c0 * ldq, ldq, nc, z, err, s);
    std::vector<float> zh(nc);
    if (e == cudaSuccess) e = cudaMemcpyAsync(zh.data(), z, nc * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(z, s);
    cudaFreeAsync(err, s);
    if (e != cudaSuccess) {
      r.tau_margin = keep;
      rc = cuda_fail(e, "rbc_router_train_with_distance: calibration");
    } else if (herr) {
      r.tau_margin = keep;
      rc = fail(RBC_ERR_ITER_LIMIT, "rbc_router_train_with_distance: a bounded device wait ran out");
    } else {
      std::vector<float> res;
      res.reserve(nc);
      for (uint64_t i = 0; i < nc; i++)
        if (std::isfinite(h[c0 + i])) res.push_back(h[c0 + i] - zh[i]);
      if (res.empty()) {
        r.tau_margin = 3.f;
      } else {
        std::sort(res.begin(), res.end());
        r.tau_margin = res[std::min<size_t>(res.size() - 1, (size_t)(0.995 * res.size()))];
      }
    }
  }
  RCK(cudaFreeAsync(dt, s));
  RCK(cudaStreamSynchronize(s));
  return rc;
}

int rbc_router_gradients_with_distance(rbc_router *router, const float *dQ, uint32_t batch, uint32_t ldq,
                                       const uint32_t *dLabels, const float *dTargets, float *loss, float *h_grads,
                                       void *stream) {
  if (!router || !dTargets || !router->r.T)
    return fail(RBC_ERR_INVALID, "rbc_router_gradients_with_distance: bad argument or no distance head");
  router->r.tau_src = dTargets;
  const int rc = rbc_router_gradients(router, dQ, batch, ldq, dLabels, loss, h_grads, stream);
  router->r.tau_src = nullptr;
  return rc;
}

int rbc_router_predict_distance(rbc_router *router, const float *dQ, uint64_t m, uint32_t ldq, const float *dNear,
                                float *dDist, void *stream) {
  if (!router || (m && (!dQ || !dDist || !dNear)))
    return fail(RBC_ERR_INVALID, "rbc_router_predict_distance: bad argument");
  Router &r = router->r;
  if (!r.T) return fail(RBC_ERR_INVALID, "rbc_router_predict_distance: the router has no distance head");
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t *err = nullptr, herr = 0;
  RCK(cudaMallocAsync(&err, 4, s));
  RCK(cudaMemsetAsync(err, 0, 4, s));
  const uint32_t chunk = 1u << 20;
  for (uint64_t i = 0; i < m; i += chunk) {
    const uint32_t b = (uint32_t)std::min<uint64_t>(chunk, m - i);
    RCK(r.predict_tau(dQ + i * ldq, ldq, b, dNear + i, dDist + i, err, s));
  }
  RCK(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s));
  RCK(cudaFreeAsync(err, s));
  RCK(cudaStreamSynchronize(s));
  if (herr) return fail(RBC_ERR_ITER_LIMIT, "rbc_router_predict_distance: a bounded device wait ran out");
  return RBC_OK;
}

int rbc_router_top_lists(rbc_router *router, const float *dQ, uint64_t m, uint32_t ldq, uint32_t P, uint32_t *dLists,
                         void *stream) {
  if (!router || (m && (!dQ || !dLists)) || P < 1 || P > 16)
    return fail(RBC_ERR_INVALID, "rbc_router_top_lists: bad argument (P in [1, 16])");
  Router &r = router->r;
  if (ldq < r.d) return fail(RBC_ERR_INVALID, "rbc_router_top_lists: ldq < d");
  if (m == 0) return RBC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t *err = nullptr, herr = 0;
  float *scratch = nullptr;
  const bool fused = r.top_ok(P);
  const uint32_t chunk = fused ? (1u << 18) : 8192;
  const size_t per = fused ? P : (size_t)P + r.L;  // probed distances (+ logits)
  RCK(cudaMallocAsync(&err, 4, s));
  RCK(cudaMemsetAsync(err, 0, 4, s));
  RCK(cudaMallocAsync(&scratch, (size_t)std::min<uint64_t>(chunk, m) * per * 4, s));
  cudaError_t e = cudaSuccess;
  for (uint64_t i = 0; i < m && e == cudaSuccess; i += chunk) {
    const uint32_t b = (uint32_t)std::min<uint64_t>(chunk, m - i);
    if (fused) {
      e = r.probes_tc(dQ + i * ldq, ldq, b, P, 0, nullptr, nullptr, dLists + i * P, scratch, err, s);
    } else {
      float *logits = scratch + (size_t)std::min<uint64_t>(chunk, m) * P;
      if (r.tc_ok()) {
        e = r.forward_tc(dQ + i * ldq, ldq, b, logits, err, s);
      } else {
        e = r.alloc_batch(std::min<uint32_t>(b, 4096), s);
        for (uint32_t j = 0; j < b && e == cudaSuccess; j += 4096)
          e = r.forward(dQ + (i + j) * ldq, ldq, std::min<uint32_t>(4096, b - j), logits + (size_t)j * r.L, s);
      }
      if (e == cudaSuccess)
        e = launch_router_probes(logits, b, r.L, P, 0, nullptr, nullptr, dLists + i * P, scratch, s);
    }
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(scratch, s);
  cudaFreeAsync(err, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_router_top_lists");
  if (herr) return fail(RBC_ERR_ITER_LIMIT, "rbc_router_top_lists: a bounded device wait ran out");
  return RBC_OK;
}

int rbc_router_distance_params(const rbc_router *router, float *mu, float *sigma, float *margin) {
  if (!router || !router->r.T) return fail(RBC_ERR_INVALID, "rbc_router_distance_params: no distance head");
  if (mu) *mu = router->r.tau_mu;
  if (sigma) *sigma = router->r.tau_sigma;
  if (margin) *margin = router->r.tau_margin;
  return RBC_OK;
}

int rbc_router_set_distance_margin(rbc_router *router, float margin) {
  if (!router || !router->r.T || !std::isfinite(margin))
    return fail(RBC_ERR_INVALID, "rbc_router_set_distance_margin: no distance head or bad margin");
  router->r.tau_margin = margin;
  return RBC_OK;
}

int rbc_router_logits(rbc_router *router, const float *dQ, uint64_t m, uint32_t ldq, float *dLogits, void *stream) {
  if (!router || (m && (!dQ || !dLogits))) return fail(RBC_ERR_INVALID, "rbc_router_logits: bad argument");
  Router &r = router->r;
  cudaStream_t s = (cudaStream_t)stream;
  if (r.tc_ok()) {  // the inference the queries use: tensor-core GEMMs
    uint32_t *err = nullptr, herr = 0;
    RCK(cudaMallocAsync(&err, 4, s));
    RCK(cudaMemsetAsync(err, 0, 4, s));
    const uint32_t chunk = 1u << 20;
    for (uint64_t i = 0; i < m; i += chunk) {
      const uint32_t b = (uint32_t)std::min<uint64_t>(chunk, m - i);
      RCK(r.forward_tc(dQ + i * ldq, ldq, b, dLogits + i * r.L, err, s));
    }
    RCK(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s));
    RCK(cudaFreeAsync(err, s));
    RCK(cudaStreamSynchronize(s));
    if (herr) return fail(RBC_ERR_ITER_LIMIT, "rbc_router_logits: a bounded device wait ran out");
    return RBC_OK;
  }
  const uint32_t chunk = 4096;
  RCK(r.alloc_batch(chunk, s));
  for (uint64_t i = 0; i < m; i += chunk) {
    const uint32_t b = (uint32_t)std::min<uint64_t>(chunk, m - i);
    RCK(r.forward(dQ + i * ldq, ldq, b, dLogits + i * r.L, s));
  }
  RCK(cudaStreamSynchronize(s));
  return RBC_OK;
}

}  // extern "C"
