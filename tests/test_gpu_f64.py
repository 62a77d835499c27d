"""The double-precision variant (the reference built with real = double,
defs.h:27-31) against the double oracle.

Ids and float64 distances must equal the oracle's bit for bit: the variant
reranks with the double build's sequential arithmetic and settles every query
its certificate cannot by a search in double.  The stated tolerance for the
distances is 1e-12 relative; assert_same also checks equality.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def assert_same(ids, dists, ref_ids, ref_dists, rbc):
    ids = rbc.u32(ids)
    dists = dists.cpu().numpy() if hasattr(dists, "cpu") else dists
    assert dists.dtype == np.float64
    np.testing.assert_array_equal(ids, ref_ids)
    np.testing.assert_allclose(dists, ref_dists, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(dists, ref_dists)


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("n,m,d,k", [(3000, 100, 16, 10), (5000, 64, 128, 32), (777, 33, 3, 1),
                                     (20000, 50, 40, 100), (2000, 30, 300, 5)])
def test_brute_knn_f64(rbc, oracle, metric, n, m, d, k):
    rng = np.random.default_rng(n + d)
    X = rng.standard_normal((n, d))
    Q = rng.standard_normal((m, d))
    ids, dists, nopen = rbc.brute_knn_f64(X, Q, k, metric)
    ri, rd = oracle.knn_f64(X, Q, k, metric)
    assert_same(ids, dists, ri, rd, rbc)
    assert nopen <= m // 10  # continuous data: the certificate settles nearly every query


@pytest.mark.parametrize("tag", ["sample", "near"])
@pytest.mark.parametrize("metric", [0, 1])
def test_f64_golden_brute_and_index(rbc, tag, metric):
    g = load_golden("f64_cases")
    mt = "l1" if metric else "l2"
    X, Q = g[f"{tag}_X"], g[f"{tag}_Q"]
    ids, dists, nopen = rbc.brute_knn_f64(X, Q, 32, metric)
    assert_same(ids, dists, g[f"{tag}_ids_{mt}"], g[f"{tag}_dists_{mt}"], rbc)
    if tag == "near":
        assert nopen > 0  # float rounding merges the points: the double search settles them
    idx = rbc.Index(X, 64, metric=metric, seed=3)
    assert idx.info()["flags"] & rbc.BUILD_F64
    ids, dists = idx.query(Q, 32)
    assert_same(ids, dists, g[f"{tag}_ids_{mt}"], g[f"{tag}_dists_{mt}"], rbc)
    if tag == "near":
        assert idx.stats()["fallback_queries"] > 0
    idx.close()


@pytest.mark.parametrize("metric", [0, 1])
@pytest.mark.parametrize("case", [
    # n, m, d, nr, k
    (30000, 300, 64, 256, 10),
    (20000, 200, 128, 200, 32),
    (9000, 111, 16, 64, 70),
])
def test_f64_index_exact(rbc, oracle, metric, case):
    n, m, d, nr, k = case
    X = rbc.synth(1, 51, 0, n, d, ncomp=100, sigma_lo=0.05, sigma_hi=0.05).double().cpu().numpy()
    Q = rbc.synth(1, 51, 1, m, d, ncomp=100, sigma_lo=0.05, sigma_hi=0.05).double().cpu().numpy()
    rng = np.random.default_rng(n)
    X += rng.standard_normal(X.shape) * 1e-9  # below float resolution
    Q += rng.standard_normal(Q.shape) * 1e-9
    idx = rbc.Index(X, nr, metric=metric, seed=5)
    ids, dists = idx.query(Q, k)
    ri, rd = oracle.knn_f64(X, Q, k, metric)
    assert_same(ids, dists, ri, rd, rbc)
    assert idx.stats()["fallback_queries"] <= m // 10
    idx.close()


def test_f64_tensor_filter(rbc, oracle):
    # integer features moved off the integers by an offset below float resolution
    X = rbc.synth(2, 52, 0, 20000, 128).double().cpu().numpy() + 1e-9
    Q = rbc.synth(2, 52, 1, 150, 128).double().cpu().numpy() + 3e-9
    idx = rbc.Index(X, 128, seed=2, flags=rbc.BUILD_PARTITION | rbc.BUILD_BF16)
    for k in (10, 40):
        ids, dists = idx.query(Q, k, mode=rbc.QUERY_EXACT_TC)
        ri, rd = oracle.knn_f64(X, Q, k)
        assert_same(ids, dists, ri, rd, rbc)
    idx.close()


def test_f64_edge_cases(rbc, oracle):
    rng = np.random.default_rng(9)
    # n < k: missing neighbours are (DBL_MAX, 0xFFFFFFFF)
    X = rng.standard_normal((20, 5))
    Q = rng.standard_normal((7, 5))
    ids, dists, _ = rbc.brute_knn_f64(X, Q, 32)
    ri, rd = oracle.knn_f64(X, Q, 32)
    assert_same(ids, dists, ri, rd, rbc)
    assert (rbc.u32(ids)[:, 20:] == 0xFFFFFFFF).all() and (dists.cpu().numpy()[:, 20:] == np.finfo(np.float64).max).all()
    idx = rbc.Index(X, 20, seed=1)
    ids, dists = idx.query(Q, 32)
    assert_same(ids, dists, ri, rd, rbc)
    idx.close()
    # duplicates and exact ties
    X = np.repeat(rng.integers(0, 4, (300, 6)).astype(np.float64), 2, axis=0)
    Q = rng.integers(0, 4, (40, 6)).astype(np.float64)
    ids, dists, _ = rbc.brute_knn_f64(X, Q, 16)
    ri, rd = oracle.knn_f64(X, Q, 16)
    assert_same(ids, dists, ri, rd, rbc)
    # values outside the float range: the brute force searches in double, the index refuses
    X = rng.standard_normal((500, 4)) * 1e30
    Q = rng.standard_normal((9, 4)) * 1e30
    ids, dists, nopen = rbc.brute_knn_f64(X, Q, 5)
    ri, rd = oracle.knn_f64(X, Q, 5)
    assert_same(ids, dists, ri, rd, rbc)
    assert nopen == 9
    with pytest.raises(rbc.RBCError):
        rbc.Index(X, 32)
    # tiny values (subnormal in float): still exact
    X = rng.standard_normal((800, 6)) * 1e-41
    Q = rng.standard_normal((10, 6)) * 1e-41
    ids, dists, _ = rbc.brute_knn_f64(X, Q, 8)
    ri, rd = oracle.knn_f64(X, Q, 8)
    assert_same(ids, dists, ri, rd, rbc)


def test_f64_range_count(rbc, oracle):
    rng = np.random.default_rng(4)
    X = rng.standard_normal((4000, 12))
    Q = rng.standard_normal((60, 12))
    for metric in (0, 1):
        _, rd = oracle.knn_f64(X, Q, 20, metric)
        ranges = rd[:, 19]
        cnt = rbc.range_count(X, Q, ranges, metric)
        np.testing.assert_array_equal(rbc.u32(cnt), oracle.range_count_f64(X, Q, ranges, metric))


def test_f64_index_api_rules(rbc, tmp_path):
    import torch
    X = np.random.default_rng(2).standard_normal((3000, 10))
    Q = X[:50] + 1e-3
    idx = rbc.Index(X, 64, seed=7)
    # a double index answers rbc_query_f64 only
    Qf = torch.zeros((1, 10), device="cuda")
    out = torch.zeros((1, 1), dtype=torch.int32, device="cuda")
    assert rbc.lib().rbc_query(idx.h, Qf.data_ptr(), 1, 10, 1, 0, out.data_ptr(), None, 1, None) == rbc.ERR_INVALID
    with pytest.raises(rbc.RBCError):
        idx.query(Q, 5, mode=rbc.QUERY_ONESHOT)
    b = rbc.Batch()
    with pytest.raises(rbc.RBCError):  # batches run the float search
        b.add(idx, torch.zeros((4, 10), device="cuda"), 5)
    b.close()
    with pytest.raises(rbc.RBCError):
        rbc.Index(X, 64, s=64, flags=rbc.BUILD_PARTITION | rbc.BUILD_ONESHOT)
    a = idx.query(Q, 12)
    p = str(tmp_path / "f64.idx")
    idx.save(p)
    idx2 = rbc.Index.load(p)
    assert idx2.f64
    b = idx2.query(Q, 12)
    assert (a[0] == b[0]).all() and (a[1] == b[1]).all()
    idx.close()
    idx2.close()
