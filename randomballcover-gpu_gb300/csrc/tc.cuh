// tc.cuh -- interface of the tensor-core (precision form) search.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace rbc {

constexpr int kShortlist = 40;  // rows kept per query by the tensor pass (4k for k = 10)

// A work unit: one 128-query tile against database rows [p0, p1), both
// multiples of 128 (the B tile height).
struct TcUnit {
  uint32_t tile;
  uint32_t pad;
  uint64_t p0, p1;
};

struct TcArgs {
  const TcUnit *units;
  uint32_t nunits;
  uint32_t kblocks;     // K / 64 (BF16 elements per 128-byte swizzled row)
  const float *xn;      // squared norm per database row (padded rows: +inf)
  uint64_t m_pad;       // query slots (multiple of 128)
  float *sl_a;          // [2][m_pad][SL] approx values (without ||q||^2), ascending
  uint32_t *sl_row;     // [2][m_pad][SL] database rows
  uint32_t *sl_sel;     // per query: which of the two buffers is current
  uint32_t *sl_theta;   // per query: largest approx kept once SL rows are held
  uint32_t *sl_lock;
  uint32_t *err;
};

struct RerankArgs {
  const float *X;        // FP32 database rows (list-major), stride ld
  const uint32_t *pid;   // row -> original id
  const float *Q;        // FP32 query rows in slot order, stride ld
  const uint32_t *order; // slot -> query index (output row); nullptr: identity
  uint32_t ld, dp, k;
  uint64_t m, m_pad;
  const float *sl_a;
  const uint32_t *sl_row;
  const uint32_t *sl_sel;
  const float *qn;
  const uint8_t *q_inexact;
  uint32_t x_inexact;
  float maxnorm;
  uint32_t *ids;
  float *dists;
  uint32_t ldo;
  uint32_t *nfail;
  uint32_t *fail;
};

// Upper bound on |approx(q,x) - exact(q,x)| for every database row x, where
// exact is the reference's sequential FP32 difference-form distance and
// approx = fl(fl(||x||^2 - 2 q.x) + ||q||^2) with q.x from BF16 operands and
// FP32 tensor-core accumulation.  Terms (u = 2^-24, b = 2^-8 the BF16 unit
// roundoff, applied only to operands that are not exact in BF16):
//   operand rounding      (b_q + b_x + b_q b_x) |q| |x|, twice (the -2 q.x)
//   accumulation          d 2^-22 sum|q_i x_i| (twice the truncating bound), twice
//   two final roundings   2u (|q|^2 + |x|^2 + 2|q||x|)
//   norms and the exact
//   distance's own error  gamma_d (|q|^2 + |x|^2) and gamma_d |q - x|^2
// The total is doubled as a margin.
__host__ __device__ inline double tc_error_bound(float qn, float maxnorm, uint32_t q_inexact, uint32_t x_inexact,
                                                 uint32_t d) {
  const double u = 5.9604644775390625e-08;
  const double b = 1.0 / 256.0;
  const double gd = (d + 2) * u / (1.0 - (d + 2) * u);
  const double bq = q_inexact ? b : 0.0, bx = x_inexact ? b : 0.0;
  const double nq = sqrt((double)qn / (1.0 - gd)), X = (double)maxnorm * (1.0 + gd);
  const double quant = bq + bx + bq * bx;
  const double accum = (double)d * 4.0 * u * (1.0 + bq) * (1.0 + bx);
  const double A = 2.0 * quant + 2.0 * accum + 4.0 * u + 2.0 * gd;
  const double B = 2.0 * gd + 2.0 * u;
  return 2.0 * (A * nq * X + B * (nq * nq + X * X));
}

bool tc_supported(uint32_t dp);
uint32_t tc_kp(uint32_t d);
size_t tc_smem_bytes(uint32_t kp);
int tc_grid();
cudaError_t tc_make_map(CUtensorMap *map, const void *ptr, uint64_t rows, uint32_t kp, uint32_t box_rows);
cudaError_t launch_to_bf16(const float *src, uint32_t ld, uint64_t rows, uint64_t rows_pad, uint32_t d,
                           uint32_t kp, void *dst, float *norm, float pad_norm, uint32_t *inexact,
                           uint32_t *maxnorm_bits, cudaStream_t s);
cudaError_t launch_row_inexact(const float *src, uint32_t ld, uint64_t rows, uint32_t d, uint8_t *flag,
                               cudaStream_t s);
cudaError_t launch_sl_init(float *sl_a, uint32_t *sl_row, uint32_t *sel, uint32_t *theta, uint32_t *lock,
                           uint64_t m, cudaStream_t s);
cudaError_t launch_tc_search(const CUtensorMap &tmA, const CUtensorMap &tmB, const TcArgs &a, int grid,
                             cudaStream_t s);
cudaError_t launch_rerank(int metric, const RerankArgs &a, cudaStream_t s);

}  // namespace rbc
