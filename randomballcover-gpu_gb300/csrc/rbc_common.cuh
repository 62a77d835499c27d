// rbc_common.cuh -- shared device helpers of the RBC engine.
//
// The distance arithmetic here is the engine's definition of a distance and
// is bit-identical to the reference's distVec (utils.cu:183-191, with DIST
// from defs.h:20-21): a float accumulator, dims visited in increasing order,
// each term (q-x)*(q-x) (L2, squared) or |q-x| (L1) rounded on its own and
// added with its own rounding.  The __f*_rn intrinsics are never contracted
// into FMA by nvcc, so no build flag can change these bits.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rbc_gb300.h"

#define RBC_DUMMY 0xFFFFFFFFu

namespace rbc {

// Largest dimensionality the list-search kernels hold in shared memory.
constexpr uint32_t kMaxDim = 512;
// Internal width of every per-query neighbour list (KMAX in defs.h:9).
constexpr int kListWidth = 32;

__host__ __device__ inline uint32_t pad16(uint32_t v) { return (v + 15u) / 16u * 16u; }
__host__ __device__ inline uint32_t pad4(uint32_t v) { return (v + 3u) / 4u * 4u; }

// One coordinate term of the distance, rounded as the reference rounds it.
template <int METRIC>
__device__ __forceinline__ float term(float q, float x) {
  float t = __fsub_rn(q, x);
  if (METRIC == RBC_L1) return fabsf(t);
  return __fmul_rn(t, t);
}

template <int METRIC>
__device__ __forceinline__ float accum(float acc, float q, float x) {
  return __fadd_rn(acc, term<METRIC>(q, x));
}

// (dist, id) lexicographic order: the tie rule of bruteCPU (brute.cu:104)
// generalised to k neighbours.
__device__ __forceinline__ bool pair_less(float da, uint32_t ia, float db, uint32_t ib) {
  return da < db || (da == db && ia < ib);
}
__device__ __forceinline__ bool pair_less(double da, uint32_t ia, double db, uint32_t ib) {
  return da < db || (da == db && ia < ib);
}

// Non-negative floats order like their bit patterns; used for atomicMin/Max.
__device__ __forceinline__ uint32_t fbits(float f) { return __float_as_uint(f); }

// The warp networks below sort (dist, id) pairs with dist a float or, for the
// double-precision variant, a double.
// Warp-wide bitonic sort of 32 (dist, id) pairs, ascending, one per lane.
template <typename D>
__device__ __forceinline__ void warp_sort32(D &d, uint32_t &id) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      D od = __shfl_xor_sync(0xffffffffu, d, j);
      uint32_t oi = __shfl_xor_sync(0xffffffffu, id, j);
      bool up = ((lane & k) == 0);
      bool lower = ((lane & j) == 0);
      // the lower lane of an ascending pair keeps the smaller element
      bool take_other = (lower == up) ? pair_less(od, oi, d, id) : pair_less(d, id, od, oi);
      if (take_other) { d = od; id = oi; }
    }
  }
}

// Sort a bitonic sequence of 32 pairs held one per lane, ascending.
template <typename D>
__device__ __forceinline__ void warp_bitonic_merge32(D &d, uint32_t &id) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 16; j > 0; j >>= 1) {
    D od = __shfl_xor_sync(0xffffffffu, d, j);
    uint32_t oi = __shfl_xor_sync(0xffffffffu, id, j);
    bool lower = ((lane & j) == 0);
    bool take_other = lower ? pair_less(od, oi, d, id) : pair_less(d, id, od, oi);
    if (take_other) { d = od; id = oi; }
  }
}

// Merge 32 unsorted candidates (one per lane, (FLT_MAX, DUMMY) for none)
// into a sorted 32-entry list held one per lane: the list keeps the 32
// smallest pairs of the union.
__device__ __forceinline__ void warp_merge_into(float &ld, uint32_t &li, float cd, uint32_t ci) {
  const int lane = threadIdx.x & 31;
  warp_sort32(cd, ci);
  float rd = __shfl_sync(0xffffffffu, cd, 31 - lane);
  uint32_t ri = __shfl_sync(0xffffffffu, ci, 31 - lane);
  if (pair_less(rd, ri, ld, li)) { ld = rd; li = ri; }
  warp_bitonic_merge32(ld, li);
}

// Lists of KW = 32 W pairs held by a warp, W per lane: entry 32 w + lane is
// register w of that lane, the whole list ascending.
constexpr int kMaxListWidth = 128;
inline uint32_t list_width_for(uint32_t k) { return k <= 32 ? 32 : (k <= 64 ? 64 : 128); }

// Merge 32 unsorted candidates (one per lane) into a sorted KW-entry list,
// keeping the KW smallest pairs.  Every entry of the first KW - 32 stays (at
// most 32 + KW - 33 pairs can precede it), so the candidates compete only with
// the last 32: u = the 32 smallest of (last block, candidates); then u is
// merged down through the earlier blocks, each merge of two sorted 32-blocks
// passing its upper half up.
template <int W, typename D>
__device__ __forceinline__ void warp_merge_into_w(D (&ld)[W], uint32_t (&li)[W], D cd, uint32_t ci) {
  const int lane = threadIdx.x & 31;
  warp_sort32(cd, ci);
  D ud = __shfl_sync(0xffffffffu, cd, 31 - lane);
  uint32_t ui = __shfl_sync(0xffffffffu, ci, 31 - lane);
  if (!pair_less(ud, ui, ld[W - 1], li[W - 1])) {
    ud = ld[W - 1];
    ui = li[W - 1];
  }
  warp_bitonic_merge32(ud, ui);
#pragma unroll
  for (int j = W - 2; j >= 0; j--) {
    const D rd = __shfl_sync(0xffffffffu, ud, 31 - lane);
    const uint32_t ri = __shfl_sync(0xffffffffu, ui, 31 - lane);
    D hd, lo_d;
    uint32_t hi, lo_i;
    if (pair_less(rd, ri, ld[j], li[j])) {
      lo_d = rd;
      lo_i = ri;
      hd = ld[j];
      hi = li[j];
    } else {
      lo_d = ld[j];
      lo_i = li[j];
      hd = rd;
      hi = ri;
    }
    warp_bitonic_merge32(lo_d, lo_i);
    warp_bitonic_merge32(hd, hi);
    ld[j + 1] = hd;
    li[j + 1] = hi;
    ud = lo_d;
    ui = lo_i;
  }
  ld[0] = ud;
  li[0] = ui;
}

// g := the KW smallest pairs of two sorted KW-entry lists g and l, sorted:
// the elementwise minimum of g and reversed l is bitonic; a bitonic merge
// over KW entries (blocks compared within the lane, then lanes by shuffles)
// sorts it.
template <int W, typename D>
__device__ __forceinline__ void warp_merge_lists_w(D (&gd)[W], uint32_t (&gi)[W], const D (&ld)[W],
                                                   const uint32_t (&li)[W]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int w = 0; w < W; w++) {
    const D rd = __shfl_sync(0xffffffffu, ld[W - 1 - w], 31 - lane);
    const uint32_t ri = __shfl_sync(0xffffffffu, li[W - 1 - w], 31 - lane);
    if (pair_less(rd, ri, gd[w], gi[w])) {
      gd[w] = rd;
      gi[w] = ri;
    }
  }
  constexpr int kLog2W = W >= 4 ? 2 : (W >= 2 ? 1 : 0);
  static_assert((1 << kLog2W) == W, "W must be 1, 2 or 4");
#pragma unroll
  for (int t = 0; t < kLog2W; t++) {
    const int jb = (W >> 1) >> t;
#pragma unroll
    for (int w = 0; w < W; w++) {
      const int p = w ^ jb;
      if (p > w && pair_less(gd[p], gi[p], gd[w], gi[w])) {
        const D td = gd[w];
        const uint32_t ti = gi[w];
        gd[w] = gd[p];
        gi[w] = gi[p];
        gd[p] = td;
        gi[p] = ti;
      }
    }
  }
#pragma unroll
  for (int w = 0; w < W; w++) warp_bitonic_merge32(gd[w], gi[w]);
}

// Error word shared by kernels that bound their waits: the first error wins.
__device__ __forceinline__ void raise_error(uint32_t *err, uint32_t code) {
  if (err) atomicCAS(err, 0u, code);
}

// Take a lock word (0 -> 1) with at most `limit` failed attempts; when they
// run out, record RBC_ERR_ITER_LIMIT and return false (never a hang).
__device__ __forceinline__ bool lock_bounded(uint32_t *lock, uint32_t limit, uint32_t *err) {
  uint32_t spins = 0;
  while (atomicCAS(lock, 0u, 1u) != 0u) {
    if (++spins > limit) {
      raise_error(err, RBC_ERR_ITER_LIMIT);
      return false;
    }
    __nanosleep(32);
  }
  return true;
}

}  // namespace rbc
