"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

Run in a checkout that can see the reference sources (the reference's own
bruteCPU, compiled into oracle/_ref, cross-checks every 1-NN column):

    python tests/golden/make_golden.py

Inputs:
  sample_db.bin / sample_queries.bin  -- the reference's sample_input files
                                         (1024 x 16 and 128 x 16 float32).
  synth_*                              -- seeded counter-based synthetic data;
                                         only the recipe and a SHA-256 of the
                                         generated bytes are stored.
Outputs are .npz files with ids (uint32) and distances (float32) sorted by
(distance, id), plus build structures for fixed representative ids.

f64_cases.npz holds the double-precision variant's fixtures (the reference
built with real = double): inputs stored as float64, ids and float64
distances from the double oracle, and the double build's own bruteCPU 1-NN.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

# (name, kind, seed, n, m, d, k, ncomp, sigma_lo, sigma_hi, num_reps)
SYNTH_CASES = [
    ("synth_uniform_c1mini", O.KIND_UNIFORM, 1, 4096, 256, 16, 32, 1, 0.0, 0.0, 64),
    ("synth_mixture_d32", O.KIND_MIXTURE, 2, 6000, 200, 32, 10, 24, 0.05, 0.05, 96),
    ("synth_geometric_d128", O.KIND_GEOMETRIC, 3, 3000, 100, 128, 10, 1, 0.0, 0.0, 50),
]


def sample_inputs():
    X = np.fromfile(os.path.join(HERE, "sample_db.bin"), np.float32).reshape(1024, 16)
    Q = np.fromfile(os.path.join(HERE, "sample_queries.bin"), np.float32).reshape(128, 16)
    return X, Q


def synth_inputs(case):
    name, kind, seed, n, m, d, k, ncomp, slo, shi, nr = case
    X = O.synth(kind, seed, 0, n, d, ncomp=ncomp, sigma_lo=slo, sigma_hi=shi)
    Q = O.synth(kind, seed, 1, m, d, ncomp=ncomp, sigma_lo=slo, sigma_hi=shi)
    return X, Q


def rep_ids_for(n, nr, seed):
    return np.random.default_rng(seed).choice(n, size=nr, replace=False).astype(np.uint32)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    O.build()
    have_ref = O.ref_available()
    X, Q = sample_inputs()
    out = {}
    for metric, tag in ((O.L2, "l2"), (O.L1, "l1")):
        ids, dists = O.knn(X, Q, 32, metric)
        out[f"ids_{tag}"], out[f"dists_{tag}"] = ids, dists
    if have_ref:
        ref1 = O.ref_brute_cpu(X, Q)
        assert (ref1 == out["ids_l2"][:, 0]).all(), "oracle disagrees with the reference's bruteCPU"
        out["ref_bruteCPU_1nn"] = ref1
    reps = rep_ids_for(1024, 128, 7)
    lists, counts, rho = O.oneshot_build(X, reps, 128)
    oids, odists = O.oneshot_query(X, reps, lists, counts, Q, 32)
    owner, odist, offsets, members, radius = O.partition(X, reps)
    out.update(rep_ids=reps, oneshot_lists=lists, oneshot_counts=counts, oneshot_rho=rho, oneshot_ids=oids,
               oneshot_dists=odists, part_owner=owner, part_offsets=offsets, part_members=members,
               part_radius=radius, db_sha=sha(X), q_sha=sha(Q))
    np.savez_compressed(os.path.join(HERE, "sample_input.npz"), **out)

    for case in SYNTH_CASES:
        name, kind, seed, n, m, d, k, ncomp, slo, shi, nr = case
        X, Q = synth_inputs(case)
        res = dict(spec=np.array([kind, seed, n, m, d, k, ncomp, nr], np.int64),
                   sigma=np.array([slo, shi], np.float32), db_sha=sha(X), q_sha=sha(Q))
        for metric, tag in ((O.L2, "l2"), (O.L1, "l1")):
            ids, dists = O.knn(X, Q, k, metric)
            res[f"ids_{tag}"], res[f"dists_{tag}"] = ids, dists
        if have_ref:
            ref1 = O.ref_brute_cpu(X, Q)
            assert (ref1 == res["ids_l2"][:, 0]).all(), f"{name}: oracle disagrees with bruteCPU"
            res["ref_bruteCPU_1nn"] = ref1
        reps = rep_ids_for(n, nr, seed + 100)
        owner, odist, offsets, members, radius = O.partition(X, reps)
        res.update(rep_ids=reps, part_offsets=offsets, part_members=members, part_radius=radius)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **res)
    f64_cases(have_ref and O.ref64_available())
    print("golden fixtures written; reference cross-check:", "yes" if have_ref else "no (reference absent)")


def f64_cases(have_ref64):
    """Double-precision fixtures.  'sample': the sample input plus offsets
    below float resolution; 'near': points 1e-7 apart around 100, which all
    round to the same float (the float shortlist cannot separate them)."""
    Xs, Qs = sample_inputs()
    ii = np.arange(1024)[:, None] * 7919 + np.arange(16)[None, :] * 104729
    jj = np.arange(128)[:, None] * 7919 + np.arange(16)[None, :] * 104729 + 3
    X1 = Xs.astype(np.float64) + ((ii % 2001) - 1000) * 2.0 ** -40
    Q1 = Qs.astype(np.float64) + ((jj % 2001) - 1000) * 2.0 ** -40
    rng = np.random.default_rng(64)
    X2 = 100.0 + 1e-7 * rng.integers(-50, 51, (600, 8)).astype(np.float64)
    Q2 = 100.0 + 1e-7 * rng.integers(-50, 51, (40, 8)).astype(np.float64)
    out = {}
    for tag, X, Q in (("sample", X1, Q1), ("near", X2, Q2)):
        out[f"{tag}_X"], out[f"{tag}_Q"] = X, Q
        for metric, mt in ((O.L2, "l2"), (O.L1, "l1")):
            ids, dists = O.knn_f64(X, Q, 32, metric)
            out[f"{tag}_ids_{mt}"], out[f"{tag}_dists_{mt}"] = ids, dists
        if have_ref64:
            ref1 = O.ref_brute_cpu_f64(X, Q)
            assert (ref1 == out[f"{tag}_ids_l2"][:, 0]).all(), f"{tag}: double oracle disagrees with bruteCPU"
            out[f"{tag}_ref_bruteCPU_1nn"] = ref1
    np.savez_compressed(os.path.join(HERE, "f64_cases.npz"), **out)


if __name__ == "__main__":
    main()
