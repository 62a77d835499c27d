"""The CPU oracle, pinned against the reference's own code and the golden files."""
import hashlib

import numpy as np
import pytest

from conftest import load_golden, sample_inputs

SYNTH = ["synth_uniform_c1mini", "synth_mixture_d32", "synth_geometric_d128"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def fp64_knn(X, Q, k, metric):
    diff = Q[:, None, :].astype(np.float64) - X[None, :, :].astype(np.float64)
    D = np.abs(diff).sum(-1) if metric == 1 else (diff * diff).sum(-1)
    return D


def test_sample_matches_golden(oracle):
    X, Q = sample_inputs()
    g = load_golden("sample_input")
    assert sha(X) == str(g["db_sha"]) and sha(Q) == str(g["q_sha"])
    for metric, tag in ((oracle.L2, "l2"), (oracle.L1, "l1")):
        ids, dists = oracle.knn(X, Q, 32, metric)
        np.testing.assert_array_equal(ids, g[f"ids_{tag}"])
        np.testing.assert_array_equal(dists, g[f"dists_{tag}"])


def test_golden_first_column_is_reference_brutecpu(oracle):
    """The committed fixtures carry the reference's bruteCPU output (brute.cu:91-112)."""
    for name in ["sample_input"] + SYNTH:
        g = load_golden(name)
        assert "ref_bruteCPU_1nn" in g, name
        np.testing.assert_array_equal(g["ids_l2"][:, 0], g["ref_bruteCPU_1nn"])


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference build not present")
def test_oracle_equals_reference_brutecpu_random(oracle):
    rng = np.random.default_rng(11)
    for n, m, d in ((777, 33, 5), (2048, 64, 16), (500, 20, 130)):
        X = rng.standard_normal((n, d)).astype(np.float32)
        Q = rng.standard_normal((m, d)).astype(np.float32)
        X[17] = X[3]  # duplicate points: the lower id must win
        np.testing.assert_array_equal(oracle.brute_1nn(X, Q), oracle.ref_brute_cpu(X, Q))
        ids, _ = oracle.knn(X, Q, 1)
        np.testing.assert_array_equal(ids[:, 0], oracle.ref_brute_cpu(X, Q))


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference build not present")
def test_distance_equals_reference_distvec(oracle):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((40, 37)).astype(np.float32) * 10
    Q = rng.standard_normal((9, 37)).astype(np.float32)
    for i in range(9):
        for j in (0, 5, 39):
            assert oracle.distance(Q[i], X[j]) == oracle.ref_dist_vec(Q, X, i, j)


@pytest.mark.parametrize("name", SYNTH)
def test_synth_matches_golden(oracle, name):
    g = load_golden(name)
    kind, seed, n, m, d, k, ncomp, nr = (int(v) for v in g["spec"])
    slo, shi = (float(v) for v in g["sigma"])
    X = oracle.synth(kind, seed, 0, n, d, ncomp=ncomp, sigma_lo=slo, sigma_hi=shi)
    Q = oracle.synth(kind, seed, 1, m, d, ncomp=ncomp, sigma_lo=slo, sigma_hi=shi)
    assert sha(X) == str(g["db_sha"]) and sha(Q) == str(g["q_sha"])
    for metric, tag in ((oracle.L2, "l2"), (oracle.L1, "l1")):
        ids, dists = oracle.knn(X, Q, k, metric)
        np.testing.assert_array_equal(ids, g[f"ids_{tag}"])
        np.testing.assert_array_equal(dists, g[f"dists_{tag}"])
    owner, odist, off, mem, rad = oracle.partition(X, g["rep_ids"])
    np.testing.assert_array_equal(off, g["part_offsets"])
    np.testing.assert_array_equal(mem, g["part_members"])
    np.testing.assert_array_equal(rad, g["part_radius"])


def test_knn_order_matches_fp64_ranking(oracle):
    """Distances within 1e-6 relative of FP64, ids in FP64 order except exact-FP32 ties."""
    rng = np.random.default_rng(5)
    X = rng.random((1500, 24), dtype=np.float32)
    Q = rng.random((40, 24), dtype=np.float32)
    for metric in (oracle.L2, oracle.L1):
        ids, dists = oracle.knn(X, Q, 16, metric)
        D = fp64_knn(X, Q, 16, metric)
        ref = np.take_along_axis(D, ids.astype(np.int64), 1)
        np.testing.assert_allclose(dists, ref, rtol=1e-6)
        assert (np.diff(dists, axis=1) >= 0).all()


def test_tie_rule_lowest_id(oracle):
    X = np.zeros((50, 4), np.float32)  # every point at the same distance
    Q = np.ones((3, 4), np.float32)
    ids, dists = oracle.knn(X, Q, 32)
    np.testing.assert_array_equal(ids, np.tile(np.arange(32, dtype=np.uint32), (3, 1)))
    assert (dists == 4.0).all()


def test_fewer_points_than_k_pads(oracle):
    X = np.arange(12, dtype=np.float32).reshape(3, 4)
    ids, dists = oracle.knn(X, X[:1], 5)
    assert list(ids[0][:3]) == [0, 1, 2]
    assert (ids[0][3:] == oracle.DUMMY).all() and (dists[0][3:] == oracle.FLT_MAX).all()


def test_oneshot_lists_are_s_nearest(oracle):
    X, Q = sample_inputs()
    g = load_golden("sample_input")
    lists, counts, rho = oracle.oneshot_build(X, g["rep_ids"], 128)
    np.testing.assert_array_equal(lists, g["oneshot_lists"])
    assert (counts == 128).all()
    for r in (0, 5, 100):
        rid = g["rep_ids"][r]
        d = np.array([oracle.distance(X[rid], X[j]) for j in range(1024)], np.float32)
        order = np.lexsort((np.arange(1024), d))
        np.testing.assert_array_equal(np.sort(order[:128]).astype(np.uint32), lists[r])


def test_partition_owner_is_nearest_rep(oracle):
    g = load_golden("sample_input")
    X, _ = sample_inputs()
    reps = g["rep_ids"]
    owner, odist, off, mem, rad = oracle.partition(X, reps)
    assert off[-1] == 1024 and (np.diff(off.astype(np.int64)) >= 0).all()
    assert sorted(mem.tolist()) == list(range(1024))
    R = X[reps]
    rep, dist = oracle.nearest_rep(X, R)
    np.testing.assert_array_equal(rep, owner)
    for r in range(len(reps)):
        seg = mem[off[r]:off[r + 1]]
        assert (np.diff(seg.astype(np.int64)) > 0).all()  # ids ascending in each list
        assert (owner[seg] == r).all()
        assert rad[r] == (odist[seg].max() if len(seg) else 0.0)


def test_geometric_table_is_exact_integer_recipe(oracle):
    T = oracle.geometric_table()
    t = 1 << 56
    for v in range(1, 256):
        t = t * 20 // 21
        assert int(T[v]) == t >> 24
    g = oracle.synth(oracle.KIND_GEOMETRIC, 3, 0, 2000, 64)
    assert g.min() == 0 and g.max() <= 255 and abs(g.mean() - 20) < 0.5
    assert (g == np.round(g)).all()


def test_range_count_matches_fp32_definition(oracle):
    X, Q = sample_inputs()
    g = load_golden("sample_input")
    ranges = g["dists_l2"][:, 9].copy()
    cnt = oracle.range_count(X, Q, ranges)
    # strictly closer than the 10th distance: at most 9, at least the ones before ties
    assert (cnt <= 9).all()
    ids = g["ids_l2"]
    assert (cnt >= (g["dists_l2"][:, :9] < ranges[:, None]).sum(1)).all()


# ------------------------------------------------------------------ double-precision variant
@pytest.mark.skipif(not __import__("oracle").ref64_available(), reason="reference double build not present")
def test_f64_oracle_equals_reference_double_build(oracle):
    """The double oracle against the reference compiled with real = double (defs.h:27-31)."""
    rng = np.random.default_rng(64)
    for n, m, d in ((901, 31, 7), (2048, 40, 16), (300, 12, 130)):
        X = rng.standard_normal((n, d))
        Q = rng.standard_normal((m, d))
        X[11] = X[2]  # duplicates: the lower id wins
        np.testing.assert_array_equal(oracle.brute_1nn_f64(X, Q), oracle.ref_brute_cpu_f64(X, Q))
        ids, _ = oracle.knn_f64(X, Q, 1)
        np.testing.assert_array_equal(ids[:, 0], oracle.ref_brute_cpu_f64(X, Q))
        for i in (0, m - 1):
            for j in (0, 11, n - 1):
                assert oracle.distance64(Q[i], X[j]) == oracle.ref_dist_vec_f64(Q, X, i, j)


def test_f64_golden(oracle):
    g = load_golden("f64_cases")
    for tag in ("sample", "near"):
        X, Q = g[f"{tag}_X"], g[f"{tag}_Q"]
        np.testing.assert_array_equal(g[f"{tag}_ids_l2"][:, 0], g[f"{tag}_ref_bruteCPU_1nn"])
        for metric, mt in ((oracle.L2, "l2"), (oracle.L1, "l1")):
            ids, dists = oracle.knn_f64(X, Q, 32, metric)
            np.testing.assert_array_equal(ids, g[f"{tag}_ids_{mt}"])
            np.testing.assert_array_equal(dists, g[f"{tag}_dists_{mt}"])


def test_f64_near_case_defeats_float_ranking(oracle):
    """In the 'near' fixture the 101 distinct coordinates round to three
    floats: the float order says almost nothing, the double order decides."""
    g = load_golden("f64_cases")
    X = g["near_X"]
    assert len(np.unique(X)) > 90 and len(np.unique(X.astype(np.float32))) <= 3
    d = g["near_dists_l2"]
    assert (d[:, 1:] >= d[:, :-1]).all() and (d[:, 0] > 0).any()


def test_f64_range_count_definition(oracle):
    rng = np.random.default_rng(5)
    X = rng.standard_normal((700, 9))
    Q = rng.standard_normal((20, 9))
    ids, dists = oracle.knn_f64(X, Q, 10)
    cnt = oracle.range_count_f64(X, Q, dists[:, 9])
    assert (cnt <= 9).all() and (cnt >= 0).all()
    cnt2 = oracle.range_count_f64(X, Q, np.nextafter(dists[:, 9], np.inf))
    assert (cnt2 >= 10).all()


def test_pruning_reciprocals_round_the_safe_way():
    """The plan's pruning bound multiplies by reciprocals of 1 + gamma, 1 - gamma
    and 1 + c; the host rounds each (after a 2^-50 nudge) so the float is on
    the safe side of the exact rational value, for every padded dimension."""
    from fractions import Fraction as Fr

    def up(v):
        f = np.float32(v)
        return np.nextafter(f, np.float32(np.inf)) if float(f) < v else f

    def down(v):
        f = np.float32(v)
        return np.nextafter(f, np.float32(0)) if float(f) > v else f

    for dp in range(4, 516, 4):
        g = (dp + 8) * 2.0 ** -23
        G = Fr(dp + 8, 2 ** 23)
        assert Fr(float(down(1.0 / (1.0 + g) * (1.0 - 2.0 ** -50)))) <= 1 / (1 + G)
        assert Fr(float(up(1.0 / (1.0 - g) * (1.0 + 2.0 ** -50)))) >= 1 / (1 - G)
        assert Fr(float(down(1.0 / (2.0 + 3.0 * g) * (1.0 - 2.0 ** -50)))) <= 1 / (2 + 3 * G)
