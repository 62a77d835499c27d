// synth.cu -- counter-based synthetic matrices, generated on the device.
//
// Every value is a pure function of (seed, stream, row, column) built from
// 64-bit integer hashing; floats are formed exactly (24-bit uniforms) and
// combined in a fixed order with separately rounded operations, so a CPU
// implementation of the same recipe produces the same bits.  Kinds:
//   uniform    U[0,1)
//   mixture    isotropic Gaussian mixture: component = hash % ncomp, mean
//              U[0,1)^d per component, sigma = lo + (hi-lo) U per component,
//              noise = 12-term Irwin-Hall sum minus 6
//   geometric  integer geometric with P(V >= v) = (20/21)^v, clipped at 255
//              (mean 20), by binary search in a 256-entry threshold table
#include <algorithm>

#include "kernels.cuh"
#include "rbc_common.cuh"

namespace rbc {

namespace {

__constant__ uint32_t c_geo[256];

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t rng(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t key = mix64(seed + 0x9E3779B97F4A7C15ull * (stream + 1));
  return mix64(key + idx);
}

__device__ __forceinline__ float u01(uint64_t seed, uint64_t stream, uint64_t idx) {
  return __fmul_rn((float)(rng(seed, stream, idx) >> 40), 5.9604644775390625e-08f);
}

__device__ __forceinline__ float normal12(uint64_t seed, uint64_t stream, uint64_t idx) {
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 12; j++) s = __fadd_rn(s, u01(seed, stream, idx * 12u + (uint64_t)j));
  return __fsub_rn(s, 6.0f);
}

__global__ void synth_kernel(int kind, uint64_t seed, uint64_t stream, uint64_t r0, uint64_t rows, uint32_t d,
                             uint32_t ld, float *__restrict__ out, uint32_t ncomp, float sigma_lo,
                             float sigma_hi) {
  uint64_t total = rows * ld;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t rr = t / ld;
    uint32_t c = (uint32_t)(t - rr * ld);
    uint64_t i = r0 + rr;
    float v = 0.f;
    if (c < d) {
      uint64_t idx = i * d + c;
      if (kind == RBC_SYNTH_UNIFORM) {
        v = u01(seed, stream, idx);
      } else if (kind == RBC_SYNTH_MIXTURE) {
        uint32_t comp = (uint32_t)(rng(seed, stream + 100, i) % ncomp);
        float sg = __fadd_rn(sigma_lo, __fmul_rn(__fsub_rn(sigma_hi, sigma_lo), u01(seed, 201, comp)));
        float mu = u01(seed, 200, (uint64_t)comp * d + c);
        float z = normal12(seed, stream, idx);
        v = __fadd_rn(mu, __fmul_rn(sg, z));
      } else {
        uint32_t u = (uint32_t)(rng(seed, stream, idx) >> 32);
        uint32_t lo = 0, hi = 255;
        while (lo < hi) {
          uint32_t mid = (lo + hi + 1) >> 1;
          if (u < c_geo[mid]) lo = mid;
          else hi = mid - 1;
        }
        v = (float)lo;
      }
    }
    out[t] = v;
  }
}

}  // namespace

// T[v] = floor(2^32 (num/den)^v) in 2^56 fixed point with exact integer steps.
void geometric_table(uint32_t num, uint32_t den, uint32_t *T) {
  uint64_t t = 1ull << 56;
  T[0] = 0xFFFFFFFFu;
  for (int v = 1; v < 256; v++) {
    t = t * num / den;
    T[v] = (uint32_t)(t >> 24);
  }
}

cudaError_t launch_synth(int kind, uint64_t seed, uint64_t stream_id, uint64_t r0, uint64_t rows, uint32_t d,
                         uint32_t ld, float *out, uint32_t ncomp, float sigma_lo, float sigma_hi,
                         cudaStream_t s) {
  if (rows == 0) return cudaSuccess;
  if (kind == RBC_SYNTH_GEOMETRIC) {
    static bool loaded = false;
    if (!loaded) {
      uint32_t T[256];
      geometric_table(20, 21, T);
      cudaError_t e = cudaMemcpyToSymbol(c_geo, T, sizeof(T));
      if (e != cudaSuccess) return e;
      loaded = true;
    }
  }
  uint64_t total = rows * ld;
  unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, 152ull * 128);
  synth_kernel<<<grid, 256, 0, s>>>(kind, seed, stream_id, r0, rows, d, ld, out, ncomp == 0 ? 1 : ncomp,
                                    sigma_lo, sigma_hi);
  return launched();
}

}  // namespace rbc
