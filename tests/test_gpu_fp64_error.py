"""Distance error against float64, per configuration shape.

The engine returns the reference's FP32 distances (sequential sum of
separately rounded terms), so every returned distance must sit within the
float summation bound of the exact (float64) distance of the same pair:
|d32 - d64| <= (d + 8) 2^-23 d64, twice the bound of a sequential float sum
of d rounded non-negative terms.  Each configuration's shape and distribution
is run at a size the oracle check finishes in seconds, in every form that
applies to it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIGS = {
    # kind, n, m, d, nr, k, ncomp, sigma_lo, sigma_hi, metric
    "uniform d16 1-NN": (0, 65536, 2048, 16, 256, 1, 1, 0.0, 0.0, 0),
    "mixture d128 32-NN": (1, 100000, 400, 128, 1024, 32, 1000, 0.05, 0.05, 0),
    "geometric d128 10-NN": (2, 200000, 300, 128, 512, 10, 1, 0.0, 0.0, 0),
    "mixture d64 k10": (1, 50000, 500, 64, 224, 10, 300, 0.05, 0.05, 0),
    "mixture sigma U[0.02,0.1] 10-NN": (1, 100000, 500, 128, 512, 10, 2000, 0.02, 0.1, 0),
    "mixture d32 L1": (1, 40000, 300, 32, 200, 10, 100, 0.05, 0.05, 1),
}


def rel_error(X, Q, ids, dists, metric):
    ids = ids.astype(np.int64)
    rows = X[ids].astype(np.float64)
    diff = rows - Q.astype(np.float64)[:, None, :]
    d64 = np.abs(diff).sum(-1) if metric == 1 else (diff * diff).sum(-1)
    d32 = dists.astype(np.float64)
    zero = d64 == 0
    assert (d32[zero] == 0).all()
    return float((np.abs(d32 - d64)[~zero] / d64[~zero]).max()) if (~zero).any() else 0.0


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_distance_error_vs_fp64(rbc, oracle, name):
    kind, n, m, d, nr, k, ncomp, slo, shi, metric = CONFIGS[name]
    X = rbc.synth(kind, 77, 0, n, d, ncomp=ncomp, sigma_lo=slo, sigma_hi=shi)
    Q = rbc.synth(kind, 77, 1, m, d, ncomp=ncomp, sigma_lo=slo, sigma_hi=shi)
    Xh, Qh = X.cpu().numpy(), Q.cpu().numpy()
    flags = rbc.BUILD_PARTITION | (rbc.BUILD_BF16 if metric == 0 else 0)
    idx = rbc.Index(X, nr, metric=metric, seed=1, flags=flags)
    modes = [rbc.QUERY_EXACT] + ([rbc.QUERY_EXACT_TC] if metric == 0 else [])
    bound = (d + 8) * 2.0 ** -23
    ri, rd = oracle.knn(Xh, Qh, k, metric)
    for mode in modes:
        ids, dists = idx.query(Q, k, mode=mode)
        ids, dists = rbc.u32(ids), dists.cpu().numpy()
        np.testing.assert_array_equal(ids, ri)
        err = rel_error(Xh, Qh, ids, dists, metric)
        assert err <= bound, (name, mode, err, bound)
    idx.close()
