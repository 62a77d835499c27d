"""Batched search and the autotuner.

rbc_batch answers many independent (index, query set) instances with one
persistent search launch per round, captured once into a CUDA graph and
replayed; every instance's answer must equal the oracle's exactly, on the
first run and on replays with new query values.  Every tuning the autotuner
can pick must keep the results exact.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def check_exact(ids, dists, X, Q, k, metric, rbc, oracle):
    rid, rd = oracle.knn(X, Q, k, metric)
    np.testing.assert_array_equal(rbc.u32(ids), rid)
    np.testing.assert_array_equal(dists.cpu().numpy(), rd)


def clustered(rng, n, d, centers=20, spread=0.2):
    C = rng.standard_normal((centers, d)).astype(np.float32) * 3
    lab = rng.integers(0, centers, n)
    return (C[lab] + spread * rng.standard_normal((n, d))).astype(np.float32)


@pytest.mark.parametrize("metric", [0, 1])
def test_batch_heterogeneous_instances(rbc, oracle, metric):
    """Instances of different sizes, dimensions, k and list counts in one launch."""
    rng = np.random.default_rng(40 + metric)
    shapes = [(3000, 16, 64, 200, 10), (5000, 37, 100, 333, 32), (2000, 128, 45, 64, 1),
              (800, 3, 30, 97, 5)]
    batch = rbc.Batch()
    cases = []
    for n, d, nr, m, k in shapes:
        X = clustered(rng, n, d)
        Q = clustered(rng, m, d)
        idx = rbc.Index(X, nr, metric=metric, seed=n)
        Qd = torch.from_numpy(Q).cuda()
        ids, dists = batch.add(idx, Qd, k)
        cases.append((idx, X, Qd, k, ids, dists))
    batch.run()
    torch.cuda.synchronize()
    for idx, X, Qd, k, ids, dists in cases:
        check_exact(ids, dists, X, Qd.cpu().numpy(), k, metric, rbc, oracle)
    # replay the captured graph with new query values in the same buffers
    for rep in range(2):
        for idx, X, Qd, k, ids, dists in cases:
            Qd.copy_(torch.from_numpy(clustered(rng, Qd.shape[0], Qd.shape[1])))
        batch.run()
        torch.cuda.synchronize()
        for idx, X, Qd, k, ids, dists in cases:
            check_exact(ids, dists, X, Qd.cpu().numpy(), k, metric, rbc, oracle)
    batch.close()
    for c in cases:
        c[0].close()


def test_batch_tensor_form_instances(rbc, oracle):
    """Tensor-form instances (RBC_QUERY_EXACT_TC) in one captured graph beside
    an FP32 one: the split operand format (float mixture), the BF16 format
    (integer features, k = 32), and rows repeated 60 times, where tied
    distances leave nearly every certificate open so the device-side
    re-search answers those queries.  Exact on the first run and on replays
    with new query values."""
    rng = np.random.default_rng(77)
    batch = rbc.Batch()
    cases = []

    def add(X, Qn, nr, k, mode, seed):
        flags = rbc.BUILD_PARTITION | (rbc.BUILD_BF16 if mode == rbc.QUERY_EXACT_TC else 0)
        idx = rbc.Index(X, nr, seed=seed, flags=flags)
        Qd = torch.from_numpy(Qn).cuda()
        ids, dists = batch.add(idx, Qd, k, mode=mode)
        cases.append((idx, X, Qd, k, ids, dists))

    add(clustered(rng, 30000, 64, centers=300, spread=0.3), clustered(rng, 300, 64, centers=300, spread=0.3), 200, 10,
        rbc.QUERY_EXACT_TC, 1)
    add(rng.integers(0, 40, (20000, 128)).astype(np.float32), rng.integers(0, 40, (257, 128)).astype(np.float32), 100,
        32, rbc.QUERY_EXACT_TC, 2)
    base = rng.standard_normal((300, 32)).astype(np.float32)
    add(np.repeat(base, 60, axis=0), rng.standard_normal((150, 32)).astype(np.float32), 64, 10, rbc.QUERY_EXACT_TC, 3)
    add(clustered(rng, 5000, 37), clustered(rng, 200, 37), 100, 5, rbc.QUERY_EXACT, 4)
    assert cases[0][0].info()["tc_format"] == rbc.TC_FP16_SPLIT and cases[1][0].info()["tc_format"] == rbc.TC_BF16
    for rep in range(3):
        if rep:
            for idx, X, Qd, k, ids, dists in cases:
                if rep == 2 and X.shape[1] == 128:
                    Qd.copy_(torch.from_numpy(rng.integers(0, 40, tuple(Qd.shape)).astype(np.float32)))
                elif rep == 2:
                    Qd.copy_(Qd[torch.randperm(Qd.shape[0], device=Qd.device)] + 0.01)
        batch.run()
        torch.cuda.synchronize()
        for idx, X, Qd, k, ids, dists in cases:
            check_exact(ids, dists, X, Qd.cpu().numpy(), k, 0, rbc, oracle)
    # the duplicate-heavy instance: the tensor form alone leaves most of its
    # certificates open (the batch answered them on the device)
    idx, X, Qd = cases[2][0], cases[2][1], cases[2][2]
    idx.query(Qd, 10, mode=rbc.QUERY_EXACT_TC)
    assert idx.stats()["fallback_queries"] > Qd.shape[0] // 2
    batch.close()
    for c in cases:
        c[0].close()


def test_batch_tensor_rounds_in_few_launches(rbc, oracle):
    """64 tensor-form instances -- both operand formats, d in {32, 64, 128},
    k in {1, 10, 32}, probe rounds with FP32 prefixes, without them (the
    tensor cores take the probed lists whole, some capped: the rest of their
    longer lists searched after the threshold update) and with lists shorter
    than the prefix -- answered by one graph whose replay launches a few dozen
    kernels (each step of the query one launch over every instance), not a
    pipeline per instance.  Exact on the first run and on a replay with new
    query values."""
    rng = np.random.default_rng(11)
    batch = rbc.Batch()
    cases = []
    for i in range(64):
        n = int(np.exp(rng.uniform(np.log(2000), np.log(30000))))
        d = int(rng.choice([32, 64, 128]))
        k = int(rng.choice([1, 10, 32]))
        m = max(2, n // 100)
        if i % 2:  # integer features: the BF16 format
            X = rng.integers(0, 30, (n, d)).astype(np.float32)
            Q = rng.integers(0, 30, (m, d)).astype(np.float32)
        else:
            X = clustered(rng, n, d, centers=50)
            Q = clustered(rng, m, d, centers=50)
        idx = rbc.Index(X, int(max(32, np.sqrt(n))), seed=i, flags=rbc.BUILD_PARTITION | rbc.BUILD_BF16)
        if i % 3 == 0:
            idx.set_tc_tuning(2, rbc.TC_PREFIX_NONE)
            if i % 2 == 0:
                idx.set_tc_probe_cap(128)  # the rest of longer probed lists in a round of its own
        elif i % 3 == 1:
            idx.set_tc_tuning(4, 64)
        Qd = torch.from_numpy(Q).cuda()
        cases.append((idx, X, Qd, k) + batch.add(idx, Qd, k, mode=rbc.QUERY_EXACT_TC))
    assert {c[0].info()["tc_format"] for c in cases} == {rbc.TC_BF16, rbc.TC_FP16_SPLIT}
    batch.run()
    torch.cuda.synchronize()
    for idx, X, Qd, k, ids, dists in cases:
        check_exact(ids, dists, X, Qd.cpu().numpy(), k, 0, rbc, oracle)
    for idx, X, Qd, k, ids, dists in cases:
        Qd.copy_(Qd[torch.randperm(Qd.shape[0], device=Qd.device)] + 1.0)
    l0 = rbc.kernel_launches()
    batch.run()
    per_replay = rbc.kernel_launches() - l0
    torch.cuda.synchronize()
    assert 0 < per_replay <= 64, per_replay
    for idx, X, Qd, k, ids, dists in cases:
        check_exact(ids, dists, X, Qd.cpu().numpy(), k, 0, rbc, oracle)
    batch.close()
    for c in cases:
        c[0].close()


def test_batch_tensor_edge_instances(rbc, oracle):
    """Tensor-form batch instances at the edges: one query, one index shared by
    two instances with different k (and probe caps on it), and an index
    whose tuner chose the plain FP32 search (it joins the FP32 instances);
    exact on the first run and on a replay."""
    rng = np.random.default_rng(21)
    batch = rbc.Batch()
    cases = []

    def add(idx, X, Q, k):
        Qd = torch.from_numpy(Q).cuda()
        cases.append((idx, X, Qd, k) + batch.add(idx, Qd, k, mode=rbc.QUERY_EXACT_TC))

    flags = rbc.BUILD_PARTITION | rbc.BUILD_BF16
    Xa = rng.integers(0, 20, (12000, 64)).astype(np.float32)
    a = rbc.Index(Xa, 60, seed=1, flags=flags)
    a.set_tc_tuning(4, rbc.TC_PREFIX_NONE)
    a.set_tc_probe_cap(100)
    add(a, Xa, rng.integers(0, 20, (1, 64)).astype(np.float32), 10)    # one query
    add(a, Xa, rng.integers(0, 20, (150, 64)).astype(np.float32), 32)  # the same index, k = 32
    Xb = clustered(rng, 9000, 32, centers=40)
    b = rbc.Index(Xb, 64, seed=2, flags=flags)
    add(b, Xb, clustered(rng, 1, 32, centers=40), 1)                   # one query, 1-NN
    Xc = rbc.synth(0, 3, 0, 20000, 16).cpu().numpy()
    c = rbc.Index(Xc, 128, seed=3, flags=flags)
    c.autotune_tc(rbc.synth(0, 3, 3, 2000, 16), 1)
    add(c, Xc, rbc.synth(0, 3, 1, 300, 16).cpu().numpy(), 1)
    for rep in range(2):
        if rep:
            for idx, X, Qd, k, ids, dists in cases:
                Qd.copy_(Qd + 1.0)
        batch.run()
        torch.cuda.synchronize()
        for idx, X, Qd, k, ids, dists in cases:
            check_exact(ids, dists, X, Qd.cpu().numpy(), k, 0, rbc, oracle)
    batch.close()
    for idx in (a, b, c):
        idx.close()


def test_batch_64_instances_config_shape(rbc, oracle):
    """The batched configuration's shape scaled down: 64 instances, n log-uniform,
    d in {32, 64, 128}, k in {1, 10, 32}, m = n / 100, Gaussian mixtures with
    100-1,000 components, each index autotuned."""
    rng = np.random.default_rng(4)
    batch = rbc.Batch()
    cases = []
    for i in range(64):
        n = int(np.exp(rng.uniform(np.log(2000), np.log(40000))))
        d = int(rng.choice([32, 64, 128]))
        k = int(rng.choice([1, 10, 32]))
        m = max(1, n // 100)
        nc = int(rng.integers(100, 1001))
        X = rbc.synth(1, 400 + i, 0, n, d, ncomp=nc, sigma_lo=0.05, sigma_hi=0.05)
        Q = rbc.synth(1, 400 + i, 1, m, d, ncomp=nc, sigma_lo=0.05, sigma_hi=0.05)
        idx = rbc.Index(X, int(max(64, 2 * np.sqrt(n))), seed=i)
        idx.autotune(Q, k)
        cases.append((idx, X, Q, k) + batch.add(idx, Q, k))
    launches = rbc.kernel_launches()
    batch.run()
    batch.run()
    torch.cuda.synchronize()
    assert rbc.kernel_launches() > launches  # replays are counted
    for idx, X, Q, k, ids, dists in cases:
        check_exact(ids, dists, X.cpu().numpy(), Q.cpu().numpy(), k, 0, rbc, oracle)
    batch.close()
    for c in cases:
        c[0].close()


def test_batch_shares_an_index(rbc, oracle):
    """The same index in several instances (many clients of one database)."""
    rng = np.random.default_rng(7)
    X = clustered(rng, 6000, 24)
    idx = rbc.Index(X, 80)
    batch = rbc.Batch()
    outs = []
    for m, k in ((100, 4), (257, 32), (1, 1)):
        Qd = torch.from_numpy(clustered(rng, m, 24)).cuda()
        outs.append((Qd, k) + batch.add(idx, Qd, k))
    batch.run()
    torch.cuda.synchronize()
    for Qd, k, ids, dists in outs:
        check_exact(ids, dists, X, Qd.cpu().numpy(), k, 0, rbc, oracle)
    batch.close()
    idx.close()


def test_batch_rejects_bad_use(rbc):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((500, 8)).astype(np.float32)
    a = rbc.Index(X, 20, metric=0)
    b = rbc.Index(X, 20, metric=1)
    Qd = torch.from_numpy(X[:10].copy()).cuda()
    batch = rbc.Batch()
    batch.add(a, Qd, 3)
    with pytest.raises(rbc.RBCError):
        batch.add(b, Qd, 3)  # metrics differ
    with pytest.raises(rbc.RBCError):
        batch.add(a, Qd, 33)  # k above the list width
    batch.run()
    with pytest.raises(rbc.RBCError):
        batch.add(a, Qd, 3)  # the batch already ran
    batch.close()
    empty = rbc.Batch()
    with pytest.raises(rbc.RBCError):
        empty.run()
    empty.close()
    a.close()
    b.close()


@pytest.mark.parametrize("d", [16, 100, 300])
def test_every_tuning_is_exact(rbc, oracle, d):
    rng = np.random.default_rng(d)
    X = clustered(rng, 20000, d)
    Q = clustered(rng, 300, d)
    idx = rbc.Index(X, 140)
    rid, rd = oracle.knn(X, Q, 10)
    for tq in (0, 1, 2, 4):
        for rows in (32, 1000, 0):
            idx.set_tuning(tq, rows)
            ids, dists = idx.query(Q, 10)
            np.testing.assert_array_equal(rbc.u32(ids), rid)
            np.testing.assert_array_equal(dists.cpu().numpy(), rd)
    with pytest.raises(rbc.RBCError):
        idx.set_tuning(3, 0)
    with pytest.raises(rbc.RBCError):
        idx.set_tuning(0, 8)
    idx.close()


def test_autotune_and_cache(rbc, oracle, tmp_path):
    rng = np.random.default_rng(11)
    X = clustered(rng, 30000, 64)
    Q = clustered(rng, 500, 64)
    cache = str(tmp_path / "tune.txt")
    idx = rbc.Index(X, 170)
    idx.autotune(Q, 10, cache_path=cache)
    lines = open(cache).read().splitlines()
    assert len(lines) == 1
    n, d, nr, k, metric, tq, rows, ms = lines[0].split()
    assert (int(n), int(d), int(nr), int(k), int(metric)) == (30000, 64, 170, 10, 0)
    assert int(tq) in (1, 2, 4) and int(rows) >= 32 and float(ms) > 0
    ids, dists = idx.query(Q, 10)
    check_exact(ids, dists, X, Q, 10, 0, rbc, oracle)
    # a second index of the same shape takes the cached choice without timing
    idx2 = rbc.Index(X, 170, seed=5)
    idx2.autotune(Q, 10, cache_path=cache)
    assert len(open(cache).read().splitlines()) == 1
    ids, dists = idx2.query(Q, 10)
    check_exact(ids, dists, X, Q, 10, 0, rbc, oracle)
    idx.close()
    idx2.close()
