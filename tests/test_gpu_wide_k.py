"""k above the reference's 32 (up to 128): lists of 64 or 128 entries in the
FP32 list search, brute force and RBC queries, against the CPU oracle.

The reference fixes k at KMAX = 32 (defs.h:9); the engine keeps lists of the
smallest width in {32, 64, 128} that holds k.  Ids and distances must equal
the oracle's bit for bit (tolerance stated for the distances: 1e-6 relative).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-6


def assert_same(ids, dists, ref_ids, ref_dists, rbc):
    ids = rbc.u32(ids)
    dists = dists.cpu().numpy() if hasattr(dists, "cpu") else dists
    np.testing.assert_array_equal(ids, ref_ids)
    np.testing.assert_allclose(dists, ref_dists, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(dists, ref_dists)


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("n,m,d,k", [(5000, 100, 16, 33), (3001, 65, 128, 64), (20000, 90, 32, 100),
                                     (4000, 40, 300, 128), (50, 20, 8, 128), (777, 33, 512, 65)])
def test_brute_knn_wide_k(rbc, oracle, metric, n, m, d, k):
    rng = np.random.default_rng(n * 7 + k)
    X = rng.standard_normal((n, d)).astype(np.float32)
    Q = rng.standard_normal((m, d)).astype(np.float32)
    ids, dists = rbc.brute_knn(X, Q, k, metric)
    rid, rd = oracle.knn(X, Q, k, metric)
    assert_same(ids, dists, rid, rd, rbc)


def test_brute_wide_k_ties(rbc, oracle):
    rng = np.random.default_rng(5)
    X = rng.integers(0, 3, (6000, 8)).astype(np.float32)  # massive exact ties
    Q = rng.integers(0, 3, (64, 8)).astype(np.float32)
    for k in (33, 64, 97, 128):
        ids, dists = rbc.brute_knn(X, Q, k)
        rid, rd = oracle.knn(X, Q, k)
        assert_same(ids, dists, rid, rd, rbc)


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("case", [
    # kind, n, m, d, nr, k, ncomp, sigma
    (1, 40000, 300, 128, 400, 64, 200, 0.05),
    (1, 30000, 257, 32, 256, 128, 100, 0.08),
    (2, 20000, 200, 128, 150, 100, 1, 0.0),   # integer data, tied distances
    (0, 9000, 111, 16, 64, 33, 1, 0.0),
])
def test_rbc_exact_wide_k(rbc, oracle, metric, case):
    kind, n, m, d, nr, k, ncomp, sg = case
    X = rbc.synth(kind, 41, 0, n, d, ncomp=ncomp, sigma_lo=sg, sigma_hi=sg)
    Q = rbc.synth(kind, 41, 1, m, d, ncomp=ncomp, sigma_lo=sg, sigma_hi=sg)
    idx = rbc.Index(X, nr, metric=metric, seed=5)
    ids, dists = idx.query(Q, k)
    ri, rd = oracle.knn(X.cpu().numpy(), Q.cpu().numpy(), k, metric)
    assert_same(ids, dists, ri, rd, rbc)
    idx.close()


def test_rbc_wide_k_edge_cases(rbc, oracle):
    rng = np.random.default_rng(12)
    # n < k (missing neighbours), single list, every point a representative
    for n, nr, k in ((90, 90, 128), (200, 1, 64), (64, 64, 100)):
        X = rng.standard_normal((n, 11)).astype(np.float32)
        Q = np.concatenate([X[:3], rng.standard_normal((25, 11)).astype(np.float32)])
        idx = rbc.Index(X, nr, seed=1)
        ids, dists = idx.query(Q, k)
        ri, rd = oracle.knn(X, Q, k)
        assert_same(ids, dists, ri, rd, rbc)
        idx.close()


def test_oneshot_wide_k(rbc, oracle):
    rng = np.random.default_rng(3)
    X = rng.integers(0, 6, (6000, 12)).astype(np.float32)
    Q = rng.integers(0, 6, (70, 12)).astype(np.float32)
    reps = rng.choice(6000, 48, replace=False).astype(np.uint32)
    idx = rbc.Index(X, 48, s=400, flags=rbc.BUILD_PARTITION | rbc.BUILD_ONESHOT, rep_ids=reps)
    rl, rc, _ = oracle.oneshot_build(X, reps, 400)
    for k in (40, 128):
        ids, dists = idx.query(Q, k, mode=rbc.QUERY_ONESHOT)
        oi, od = oracle.oneshot_query(X, reps, rl, rc, Q, k)
        assert_same(ids, dists, oi, od, rbc)
    idx.close()


def test_tensor_mode_wide_k_takes_fp32_search(rbc, oracle):
    X = rbc.synth(2, 13, 0, 20000, 128)
    Q = rbc.synth(2, 13, 1, 150, 128)
    idx = rbc.Index(X, 128, seed=2, flags=rbc.BUILD_PARTITION | rbc.BUILD_BF16)
    ids, dists = idx.query(Q, 80, mode=rbc.QUERY_EXACT_TC)
    ri, rd = oracle.knn(X.cpu().numpy(), Q.cpu().numpy(), 80)
    assert_same(ids, dists, ri, rd, rbc)
    assert idx.stats()["fallback_queries"] == 0
    idx.close()


def test_wide_k_prefix_equals_narrow_k(rbc):
    # the first 32 columns of a k = 128 answer are the k = 32 answer
    X = rbc.synth(1, 17, 0, 30000, 64, ncomp=100, sigma_lo=0.05, sigma_hi=0.05)
    Q = rbc.synth(1, 17, 1, 500, 64, ncomp=100, sigma_lo=0.05, sigma_hi=0.05)
    idx = rbc.Index(X, 256, seed=3)
    a_ids, a_d = idx.query(Q, 32)
    b_ids, b_d = idx.query(Q, 128)
    assert (b_ids[:, :32] == a_ids).all() and (b_d[:, :32] == a_d).all()
    assert (b_d[:, 1:] >= b_d[:, :-1]).all()
    idx.close()


def test_k_limits(rbc):
    X = rbc.synth(0, 1, 0, 1000, 16)
    idx = rbc.Index(X, 32)
    with pytest.raises(rbc.RBCError):
        idx.query(X[:10], rbc.K_LIMIT + 1)
    with pytest.raises(rbc.RBCError):
        rbc.brute_knn(X, X[:10], rbc.K_LIMIT + 1)
    b = rbc.Batch()
    with pytest.raises(rbc.RBCError):
        b.add(idx, X[:10].contiguous(), rbc.KMAX + 1)  # batches keep the reference's 32
    b.close()
    idx.close()
