"""rbc_brute_knn_noalloc: the brute-force k-NN entry point for callers that
cannot allocate device memory at call time (a service whose GPU memory is
reserved up front by its own allocator, a latency-bound caller that must not
wait on an allocator, code running inside another allocator's callback).

It is called through the C ABI and checked against the CPU oracle: ids
bit-exact, distances within 1e-6 relative (bit-exact in practice), on two
calls in a row, so the second call proves the shared working array is reset
between calls.  A call must also leave the device's free memory and its
stream-ordered pool untouched.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-6
DUMMY = 0xFFFFFFFF


def call_noalloc(rbc, X, Q, k, metric, out=None, sync=True):
    import torch
    m = Q.shape[0]
    if out is None:
        out = (torch.full((max(m, 1), k), -7, dtype=torch.int32, device="cuda"),
               torch.full((max(m, 1), k), -7.0, dtype=torch.float32, device="cuda"))
    ids, dists = out
    rc = rbc.lib().rbc_brute_knn_noalloc(X.data_ptr(), X.shape[0], X.stride(0), Q.data_ptr(), m, Q.stride(0),
                                         X.shape[1], k, metric, ids.data_ptr(), dists.data_ptr(), k,
                                         torch.cuda.current_stream().cuda_stream)
    rbc.check(rc)
    if sync:
        torch.cuda.synchronize()
    return ids, dists


@pytest.mark.parametrize("metric", [0, 1])
def test_noalloc_matches_oracle_twice(rbc, oracle, metric):
    import torch
    cases = [(20000, 1000, 64, 32, 3), (7001, 123, 16, 10, 4)]  # second call: different m, n, d, k
    for n, m, d, k, seed in cases:
        rng = np.random.default_rng(seed + 10 * metric)
        Xh = rng.standard_normal((n, d)).astype(np.float32)
        Qh = rng.standard_normal((m, d)).astype(np.float32)
        Xh[5] = Xh[11]  # a duplicate row: the lower id first
        ids, dists = call_noalloc(rbc, torch.from_numpy(Xh).cuda(), torch.from_numpy(Qh).cuda(), k, metric)
        ref_ids, ref_dists = oracle.knn(Xh, Qh, k, metric)
        np.testing.assert_array_equal(rbc.u32(ids), ref_ids)
        np.testing.assert_allclose(dists.cpu().numpy(), ref_dists, rtol=RTOL, atol=0)


def test_noalloc_empty_database_and_empty_batch(rbc):
    """n = 0: every slot is empty (id 0xFFFFFFFF, distance FLT_MAX).  m = 0:
    the start-up call, which returns without touching the outputs."""
    import torch
    X = torch.zeros((0, 16), device="cuda")
    Q = torch.ones((5, 16), device="cuda")
    ids, dists = call_noalloc(rbc, X, Q, 4, 0)
    assert (rbc.u32(ids) == DUMMY).all()
    assert (dists.cpu().numpy() == np.finfo(np.float32).max).all()
    ids, dists = call_noalloc(rbc, X, Q[:0], 4, 0)
    assert (ids == -7).all() and (dists == -7.0).all()


def _driver():
    """The CUDA driver library (always present where a GPU is) for the memory
    counters: free device memory and the default stream-ordered pool."""
    try:
        return C.CDLL("libcuda.so.1")
    except OSError:
        pytest.skip("libcuda.so.1 not found")


def test_noalloc_call_allocates_nothing(rbc, oracle):
    """After the start-up call and one warm call, a further call leaves the
    device's free memory unchanged and the default pool's in-use high-water
    mark (reset just before it) at its current value: no allocation, not even
    a transient stream-ordered one."""
    import torch
    cu = _driver()
    USED_CURRENT, USED_HIGH = 7, 8  # CU_MEMPOOL_ATTR_USED_MEM_CURRENT / _HIGH
    dev = C.c_int()
    assert cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()) == 0
    pool = C.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0

    def pool_attr(a):
        v = C.c_uint64()
        assert cu.cuMemPoolGetAttribute(pool, a, C.byref(v)) == 0
        return v.value

    def free_bytes():
        f, t = C.c_size_t(), C.c_size_t()
        assert cu.cuMemGetInfo_v2(C.byref(f), C.byref(t)) == 0
        return f.value

    rng = np.random.default_rng(21)
    Xh = rng.standard_normal((30000, 32)).astype(np.float32)
    Qh = rng.standard_normal((2000, 32)).astype(np.float32)
    X, Q = torch.from_numpy(Xh).cuda(), torch.from_numpy(Qh).cuda()
    out = (torch.empty((2000, 10), dtype=torch.int32, device="cuda"),
           torch.empty((2000, 10), dtype=torch.float32, device="cuda"))
    call_noalloc(rbc, X, Q[:0], 10, 0)       # start-up call
    call_noalloc(rbc, X, Q, 10, 0, out=out)  # warm call
    torch.cuda.synchronize()
    free0 = free_bytes()
    zero = C.c_uint64(0)
    assert cu.cuMemPoolSetAttribute(pool, USED_HIGH, C.byref(zero)) == 0  # resets to the current use
    used0 = pool_attr(USED_CURRENT)
    ids, dists = call_noalloc(rbc, X, Q, 10, 0, out=out)
    assert pool_attr(USED_HIGH) == used0, "a stream-ordered allocation happened during the call"
    assert pool_attr(USED_CURRENT) == used0
    assert free_bytes() == free0, "device memory changed across the call"
    ref_ids, ref_dists = oracle.knn(Xh, Qh, 10)
    np.testing.assert_array_equal(rbc.u32(ids), ref_ids)
    np.testing.assert_allclose(dists.cpu().numpy(), ref_dists, rtol=RTOL, atol=0)


def test_noalloc_rejects_sizes_beyond_its_limits(rbc):
    import torch
    X = torch.zeros((100, 16), device="cuda")
    Q = torch.zeros((8193, 16), device="cuda")
    with pytest.raises(rbc.RBCError) as e:
        call_noalloc(rbc, X, Q, 5, 0)
    assert e.value.code == rbc.ERR_UNSUPPORTED and b"8192" in rbc.lib().rbc_last_error()
    X6 = torch.zeros((100, 6), device="cuda")
    with pytest.raises(rbc.RBCError) as e:
        call_noalloc(rbc, X6, X6[:4], 5, 0)
    assert e.value.code == rbc.ERR_UNSUPPORTED
