// selftest.cu -- the failure path of the bounded waits, exercised without a
// fault.  Every wait in the engine's kernels (on an mbarrier, a lock, a
// shortlist) is bounded: when it runs out it records RBC_ERR_ITER_LIMIT in
// the call's error word and returns, so the kernel ends, the context stays
// usable and the host reports the status.  rbc_selftest_bounded_wait runs
// the two wait helpers on conditions that never come true -- an mbarrier
// nobody arrives on, a lock word nobody releases -- with short limits, and
// hands back the error words they left.
#include "engine.cuh"
#include "sm100.cuh"

namespace rbc {
namespace {

__global__ void mbar_never_kernel(uint32_t *err, uint64_t limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    sm100::mbar_init(&bar, 1);
    sm100::fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) sm100::mbar_wait_for(&bar, 0, err, limit_ns);  // nothing arrives: runs out
}

__global__ void lock_never_kernel(uint32_t *lock, uint32_t *err, uint32_t limit) {
  if (threadIdx.x == 0 && lock_bounded(lock, limit, err)) atomicExch(lock, 0u);
}

}  // namespace
}  // namespace rbc

extern "C" int rbc_selftest_bounded_wait(uint32_t *mbar_status, uint32_t *lock_status, void *stream) {
  using namespace rbc;
  if (!mbar_status || !lock_status) return fail(RBC_ERR_INVALID, "rbc_selftest_bounded_wait: NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf w;
  cudaError_t e = w.alloc(16, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.p, 0, 16, s);
  uint32_t *words = w.as<uint32_t>();  // [0] mbarrier error, [1] lock error, [2] the held lock
  const uint32_t held = 1;
  if (e == cudaSuccess) e = cudaMemcpyAsync(words + 2, &held, 4, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_selftest_bounded_wait: buffers");
  mbar_never_kernel<<<1, 32, 0, s>>>(words, 50000000ull);  // 50 ms
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_selftest_bounded_wait: mbarrier wait");
  lock_never_kernel<<<1, 32, 0, s>>>(words + 2, words + 1, 1u << 14);
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_selftest_bounded_wait: lock wait");
  uint32_t h[2] = {0, 0};
  e = cudaMemcpyAsync(h, words, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_selftest_bounded_wait: status read");
  *mbar_status = h[0];
  *lock_status = h[1];
  return RBC_OK;
}
