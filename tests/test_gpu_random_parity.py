"""Randomized parity: the tensor form, the plain exact RBC, k above 32 and the
double-precision brute force against the oracle over seeded random shapes,
distributions and tuning knobs (probed lists, the FP32 / tensor split of the
probe round).  Ids and distances must equal the oracle's bit for bit."""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [101, 202])
def test_random_shapes_equal_oracle(rbc, oracle, seed, monkeypatch):
    rng = random.Random(seed)
    for it in range(24):
        kind = rng.choice([0, 1, 2])
        n, d = rng.randint(2000, 50000), rng.choice([8, 16, 32, 64, 100, 128])
        nr, m, k = rng.randint(10, 300), rng.randint(10, 400), rng.choice([1, 5, 10, 20, 32])
        monkeypatch.setenv("RBC_TC_PROBE_ROWS", rng.choice(["0", "200", "8192", "100000"]))
        monkeypatch.setenv("RBC_TC_PROBES", rng.choice(["1", "2", "4", "8"]))
        s = rng.randint(1, 10000)
        ncomp = rng.randint(5, 200)
        X = rbc.synth(kind, s, 0, n, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
        Q = rbc.synth(kind, s, 1, m, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
        Xc, Qc = X.cpu().numpy(), Q.cpu().numpy()
        ri, rd = oracle.knn(Xc, Qc, k)
        idx = rbc.Index(X, nr, seed=s, flags=rbc.BUILD_PARTITION | rbc.BUILD_BF16)
        for mode in (rbc.QUERY_EXACT_TC, rbc.QUERY_EXACT):
            ids, dists = idx.query(Q, k, mode=mode)
            case = f"iteration {it}: kind={kind} n={n} d={d} nr={nr} m={m} k={k} mode={mode}"
            np.testing.assert_array_equal(rbc.u32(ids), ri, err_msg=case)
            np.testing.assert_array_equal(dists.cpu().numpy(), rd, err_msg=case)
        idx.close()
        if it % 4 == 0:
            kk = rng.choice([33, 64, 128])
            ids, dists = rbc.brute_knn(X, Q, kk)
            wi, wd = oracle.knn(Xc, Qc, kk)
            np.testing.assert_array_equal(rbc.u32(ids), wi)
            np.testing.assert_array_equal(dists.cpu().numpy(), wd)
            X64 = Xc.astype(np.float64) + np.random.default_rng(s).standard_normal(Xc.shape) * 1e-9
            Q64 = Qc.astype(np.float64)
            i64, d64, _ = rbc.brute_knn_f64(X64, Q64, k)
            oi, od = oracle.knn_f64(X64, Q64, k)
            np.testing.assert_array_equal(rbc.u32(i64), oi)
            np.testing.assert_array_equal(d64.cpu().numpy(), od)
