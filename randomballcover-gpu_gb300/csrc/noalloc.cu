// noalloc.cu -- brute-force exact k-NN that allocates no memory.
//
// rbc_brute_knn obtains its working buffers (per-query neighbour lists,
// thresholds, locks, the work list) from the stream-ordered allocator on every
// call.  Some callers cannot allocate at call time: a service that reserves
// its whole GPU memory budget up front (a framework's caching allocator owns
// the rest of the device, so an extra cudaMalloc can fail or fragment it), a
// latency-bound caller that must not take the allocator's locks or pay its
// unpredictable cost on the query path, or code that runs from inside another
// allocator's callback and must not re-enter it.  rbc_brute_knn_noalloc serves
// them: it runs the same search kernel with its working buffers in one
// file-scope device array of fixed size instead.
//
// Limits and rules:
//   * at most kNoAllocMaxQueries (8192) queries per call, d a multiple of 4
//     and at most 512, X and Q sharing one row stride (a multiple of 4 floats)
//     and 16-byte aligned: the kernel reads the caller's rows directly
//     instead of copying them into padded buffers;
//   * the array (about 2.4 MB) is part of this library's device code; CUDA
//     loads that code on each device lazily, so the array takes device
//     memory at the first call on a device and keeps it until the process
//     exits.  A call with m = 0 does exactly that and nothing else: make one
//     at start-up on every device, while memory is still free and before any
//     stream capture (it also looks the array's device address up with
//     cudaGetSymbolAddress);
//   * the address is looked up again when the device's context changes
//     (after cudaDeviceReset, say);
//   * all calls share the array: calls that overlap on the GPU (different
//     streams or threads without ordering between them) race and corrupt each
//     other's results.  Order them on one stream, or serialise them.
#include <cuda.h>

#include <mutex>

#include "engine.cuh"
#include "kernels.cuh"
#include "rbc_common.cuh"

namespace {

constexpr uint64_t kNoAllocMaxQueries = 8192;
constexpr uint64_t kNoAllocMaxItems = 8192;

// Layout of the array: per-query lists (dist, id), thresholds, locks, the
// query index of every slot, the work items, and the control words.
constexpr size_t kResD = 0;
constexpr size_t kResI = kResD + kNoAllocMaxQueries * rbc::kListWidth * 4;
constexpr size_t kTau = kResI + kNoAllocMaxQueries * rbc::kListWidth * 4;
constexpr size_t kLock = kTau + kNoAllocMaxQueries * 4;
constexpr size_t kQidx = kLock + kNoAllocMaxQueries * 4;
constexpr size_t kItems = kQidx + kNoAllocMaxQueries * 4;
constexpr size_t kCtl = kItems + kNoAllocMaxItems * sizeof(rbc::SearchItem);
constexpr size_t kScratchBytes = kCtl + 256;

}  // namespace

// The working memory of every rbc_brute_knn_noalloc call on a device.  In host
// code this name is only a stand-in for the symbol: its device address comes
// from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace rbc {

namespace {

std::mutex g_mu;
// Per device: the array's address and the id of the context it belongs to.
struct ScratchSlot {
  void *addr = nullptr;
  unsigned long long ctx = 0;
};
ScratchSlot g_slot[64];

// Unique id of the calling thread's current context (driver entry points
// found at run time, so the library needs no link to the driver); false when
// there is none or the driver lacks the calls.
bool current_context_id(unsigned long long *id) {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool tried = false;
  if (!tried) {
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void **)&get_current, 4000, cudaEnableDefault, &q1) !=
            cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess)
      get_current = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", (void **)&get_id, 12000, cudaEnableDefault, &q2) !=
            cudaSuccess ||
        q2 != cudaDriverEntryPointSuccess)
      get_id = nullptr;
    tried = true;
  }
  CUcontext c = nullptr;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c) return false;
  return get_id(c, id) == CUDA_SUCCESS;
}

// Device address of the array on the current device: looked up once per
// device and context, with that device current.
int scratch_address(unsigned char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_brute_knn_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(RBC_ERR_UNSUPPORTED, "rbc_brute_knn_noalloc: device index above 63");
  std::lock_guard<std::mutex> lk(g_mu);
  ScratchSlot &slot = g_slot[dev];
  unsigned long long ctx = 0;
  const bool known = current_context_id(&ctx);
  if (!slot.addr || !known || ctx != slot.ctx) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(e, "rbc_brute_knn_noalloc: cudaGetSymbolAddress");
    slot.addr = p;
    slot.ctx = current_context_id(&ctx) ? ctx : 0;
  }
  *out = static_cast<unsigned char *>(slot.addr);
  return RBC_OK;
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

}  // namespace rbc

using namespace rbc;

extern "C" int rbc_brute_knn_noalloc(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m,
                                     uint32_t ldq, uint32_t d, uint32_t k, int metric, uint32_t *dIds,
                                     float *dDists, uint32_t ldo, void *stream) {
  if (k < 1 || k > (uint32_t)kListWidth) return fail(RBC_ERR_INVALID, "rbc_brute_knn_noalloc: k must be in [1, 32]");
  if (ldo < k) return fail(RBC_ERR_INVALID, "rbc_brute_knn_noalloc: ldo < k");
  if (metric != RBC_L2 && metric != RBC_L1) return fail(RBC_ERR_INVALID, "rbc_brute_knn_noalloc: unknown metric");
  unsigned char *scr = nullptr;
  if (m == 0) return scratch_address(&scr);  // the start-up call: the array is taken and found, nothing else
  if (m > kNoAllocMaxQueries)
    return fail(RBC_ERR_UNSUPPORTED, "rbc_brute_knn_noalloc: more than 8192 queries per call (split the batch)");
  if (!dQ || (!dIds && !dDists) || (n && !dX)) return fail(RBC_ERR_INVALID, "rbc_brute_knn_noalloc: NULL buffer");
  if (n >= 0xFFFFFFFFull) return fail(RBC_ERR_INVALID, "rbc_brute_knn_noalloc: n must be below 2^32-1");
  if (d == 0 || d % 4 != 0 || d > kMaxDim)
    return fail(RBC_ERR_UNSUPPORTED, "rbc_brute_knn_noalloc: d must be a multiple of 4 in [4, 512]");
  if (ldx != ldq || ldx < d || ldx % 4 != 0)
    return fail(RBC_ERR_UNSUPPORTED, "rbc_brute_knn_noalloc: X and Q must share a row stride that is a multiple of 4");
  if (!aligned16(dX) || !aligned16(dQ))
    return fail(RBC_ERR_UNSUPPORTED, "rbc_brute_knn_noalloc: X and Q must be 16-byte aligned");

  int rc = scratch_address(&scr);
  if (rc != RBC_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t qtile = (uint32_t)search_query_tile(d);
  const int grid = search_grid(metric, d);
  const uint64_t qtiles = (m + qtile - 1) / qtile;
  uint64_t nchunks = (4ull * grid + qtiles - 1) / qtiles;
  if (nchunks < 1) nchunks = 1;
  if (n / 256 < nchunks) nchunks = n / 256 ? n / 256 : 1;
  if (nchunks * qtiles > kNoAllocMaxItems) nchunks = kNoAllocMaxItems / qtiles;
  uint32_t chunk = (uint32_t)(((n + nchunks - 1) / nchunks + 31) / 32 * 32);
  if (chunk == 0) chunk = 32;

  float *res_d = reinterpret_cast<float *>(scr + kResD);
  uint32_t *res_i = reinterpret_cast<uint32_t *>(scr + kResI);
  uint32_t *tau = reinterpret_cast<uint32_t *>(scr + kTau);
  uint32_t *lock = reinterpret_cast<uint32_t *>(scr + kLock);
  uint32_t *qidx = reinterpret_cast<uint32_t *>(scr + kQidx);
  SearchItem *items = reinterpret_cast<SearchItem *>(scr + kItems);
  uint32_t *ctl = reinterpret_cast<uint32_t *>(scr + kCtl);  // [0] work, [1] items, [2] error

  // the array keeps the previous call's contents: reset what must start at zero
  cudaError_t e = cudaMemsetAsync(ctl, 0, 64, s);
  if (e == cudaSuccess) e = launch_init_results(res_d, res_i, tau, lock, m, kListWidth, s);
  if (e == cudaSuccess) e = launch_brute_items(items, ctl + 1, qidx, n, chunk, m, qtile, s);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_brute_knn_noalloc: set-up launches");
  SearchArgs sa{};
  sa.X = dX;
  sa.pid = nullptr;
  sa.Q = dQ;
  sa.qidx = qidx;
  sa.qthr = nullptr;
  sa.items = items;
  sa.nitems = ctl + 1;
  sa.work = ctl;
  sa.res_d = res_d;
  sa.res_i = res_i;
  sa.tau = tau;
  sa.lock = lock;
  sa.err = ctl + 2;
  sa.stats = nullptr;
  sa.ld = ldx;
  sa.dp = d;
  sa.k = k;
  if (n) {
    e = launch_search(metric, sa, grid, s);
    if (e != cudaSuccess) return cuda_fail(e, "rbc_brute_knn_noalloc: search launch");
  }
  e = launch_write_results(res_d, res_i, m, k, kListWidth, dIds, dDists, ldo, s);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_brute_knn_noalloc: result launch");
  uint32_t err_word = 0;
  e = cudaMemcpyAsync(&err_word, ctl + 2, sizeof(err_word), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_brute_knn_noalloc: completion");
  if (err_word) return fail((int)err_word, "rbc_brute_knn_noalloc: a bounded device wait ran out");
  return RBC_OK;
}
