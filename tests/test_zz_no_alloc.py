"""rbc_brute_knn_noalloc: the brute-force k-NN entry point for callers that
cannot allocate device memory at call time (a service whose GPU memory is
reserved up front by its own allocator, a latency-bound caller that must not
wait on an allocator, code running inside another allocator's callback).

It is called through the C ABI and must return what rbc_brute_knn returns:
ids bit-exact, distances within 1e-6 relative (bit-exact in practice), on
two calls in a row, so the second call proves the shared working array is
reset between calls.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-6


def call_noalloc(rbc, X, Q, k, metric):
    import torch
    m = Q.shape[0]
    ids = torch.full((m, k), -7, dtype=torch.int32, device="cuda")
    dists = torch.full((m, k), -7.0, dtype=torch.float32, device="cuda")
    rc = rbc.lib().rbc_brute_knn_noalloc(X.data_ptr(), X.shape[0], X.stride(0), Q.data_ptr(), m, Q.stride(0),
                                         X.shape[1], k, metric, ids.data_ptr(), dists.data_ptr(), k,
                                         torch.cuda.current_stream().cuda_stream)
    rbc.check(rc)
    torch.cuda.synchronize()
    return ids, dists


@pytest.mark.parametrize("metric", [0, 1])
def test_noalloc_matches_brute_knn_twice(rbc, metric):
    import torch
    cases = [(20000, 1000, 64, 32, 3), (7001, 123, 16, 10, 4)]  # second call: different m, n, d, k
    for n, m, d, k, seed in cases:
        rng = np.random.default_rng(seed + 10 * metric)
        X = torch.from_numpy(rng.standard_normal((n, d)).astype(np.float32)).cuda()
        Q = torch.from_numpy(rng.standard_normal((m, d)).astype(np.float32)).cuda()
        ids, dists = call_noalloc(rbc, X, Q, k, metric)
        ref_ids, ref_dists = rbc.brute_knn(X, Q, k, metric)
        np.testing.assert_array_equal(rbc.u32(ids), rbc.u32(ref_ids))
        np.testing.assert_allclose(dists.cpu().numpy(), ref_dists.cpu().numpy(), rtol=RTOL, atol=0)


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
