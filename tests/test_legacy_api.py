"""The reference's C++ API as a drop-in: programs written for it compile
against include/ and link against librbcgb.so; on the GPU they return the
oracle's neighbours."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, load_golden, sample_inputs

INCLUDE = os.path.join(ROOT, "include")
REF_SRC = __import__("oracle").ref_dir()  # the reference's sources, where this machine has them
REF_DRIVER = os.path.join(REF_SRC, "driver.cu") if REF_SRC else ""


def compile_program(src, out, engine_lib, extra=(), lib="rbcgb"):
    libdir = os.path.dirname(engine_lib.LIB_PATH)
    cmd = ["nvcc", "-O2", "-std=c++17", *extra, f"-I{INCLUDE}", src, "-o", out, f"-L{libdir}", f"-l{lib}",
           f"-Xlinker=-rpath={libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference sources not present")
def test_reference_driver_links_against_engine(engine_lib, tmp_path):
    """The reference's own driver.cu and headers, unmodified, linked to this
    engine: every C++ symbol it calls resolves in librbcgb.so.  The two
    defines map runtime calls CUDA 13 removed (the reference targets CUDA 3)."""
    compile_program(REF_DRIVER, str(tmp_path / "testRBC"), engine_lib,
                    extra=("-DcudaThreadExit=cudaDeviceReset", "-DcudaThreadSynchronize=cudaDeviceSynchronize"))


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference sources not present")
def test_reference_driver_compiles_against_engine_headers(engine_lib, tmp_path):
    """The same driver source compiled against this engine's include/ only."""
    src = tmp_path / "driver.cu"
    src.write_bytes(open(REF_DRIVER, "rb").read())
    compile_program(str(src), str(tmp_path / "testRBC2"), engine_lib)


def test_legacy_driver_compiles(engine_lib, tmp_path):
    compile_program(os.path.join(ROOT, "tests", "legacy_driver.cu"), str(tmp_path / "legacy_driver"), engine_lib)


@pytest.mark.gpu
def test_legacy_driver_on_sample_input(engine_lib, rbc, tmp_path):
    exe = compile_program(os.path.join(ROOT, "tests", "legacy_driver.cu"), str(tmp_path / "legacy_driver"),
                          engine_lib)
    outs = [str(tmp_path / f) for f in ("rbc.bin", "brute.bin", "nn1.bin")]
    r = subprocess.run([exe, os.path.join(GOLDEN, "sample_db.bin"), os.path.join(GOLDEN, "sample_queries.bin"),
                        "1024", "128", "16", "128"] + outs, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "one-shot list entries: 16384" in r.stdout  # 128 reps x s = 128, as the reference's dxMap
    g = load_golden("sample_input")
    for path in outs[:2]:
        raw = np.fromfile(path, np.uint8)
        ids = raw[: 128 * 32 * 4].view(np.uint32).reshape(128, 32)
        dists = raw[128 * 32 * 4:].view(np.float32).reshape(128, 32)
        np.testing.assert_array_equal(ids, g["ids_l2"])
        np.testing.assert_array_equal(dists, g["dists_l2"])
    nn = np.fromfile(outs[2], np.uint32)
    for j in range(3):
        np.testing.assert_array_equal(nn[j * 128:(j + 1) * 128], g["ref_bruteCPU_1nn"])
    np.testing.assert_array_equal(nn[384:].view(np.float32), g["dists_l2"][:, 0])


def test_legacy_plan_driver_compiles(engine_lib, tmp_path):
    """The plan functions of the reference's rbc.h (initCompPlan, freeCompPlan,
    computeNNs, computeKNNs) link, in both builds."""
    src = os.path.join(ROOT, "tests", "legacy_plan_driver.cu")
    compile_program(src, str(tmp_path / "plan"), engine_lib)
    compile_program(src, str(tmp_path / "plan64"), engine_lib, extra=("-DRBC_REAL_DOUBLE",), lib="rbcgb_f64")


def _plan_oracle(oracle, X, Q, members_of, k=32):
    """For every query, the oracle's k-NN over the database rows members_of(i)
    (increasing ids, repeats kept), as (ids, dists) under (distance, id)."""
    ids = np.full((Q.shape[0], k), oracle.DUMMY, np.uint32)
    dists = np.full((Q.shape[0], k), oracle.FLT_MAX, np.float32)
    for i in range(Q.shape[0]):
        mem = members_of(i)
        if len(mem) == 0:
            continue
        pos, dd = oracle.knn(np.ascontiguousarray(X[mem]), np.ascontiguousarray(Q[i:i + 1]), k)
        ok = pos[0] != oracle.DUMMY
        ids[i, ok] = mem[pos[0][ok]]
        dists[i, ok] = dd[0][ok]
    return ids, dists


@pytest.mark.gpu
def test_plan_api_on_sample_input(engine_lib, rbc, oracle, tmp_path):
    """The reference's kqueryRBC / queryRBC steps run one by one (rbc.cu:19-123)
    through initCompPlan + computeKNNs / computeNNs: under the identity
    computation matrix each query gets the oracle's 32-NN over its nearest
    representative's one-shot list, under the full matrix over every list
    (rows in several lists count once per list), and computeNNs the first of
    the identity answer."""
    exe = compile_program(os.path.join(ROOT, "tests", "legacy_plan_driver.cu"), str(tmp_path / "plan"), engine_lib)
    out = str(tmp_path / "plan.bin")
    m, nr = 128, 128
    r = subprocess.run([exe, os.path.join(GOLDEN, "sample_db.bin"), os.path.join(GOLDEN, "sample_queries.bin"),
                        "1024", str(m), "16", str(nr), out], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, np.uint8)
    off = 0

    def take(count, dt):
        nonlocal off
        a = raw[off:off + 4 * count].view(dt)
        off += 4 * count
        return a

    rep = take(m, np.uint32)
    lists = take(nr * nr, np.uint32).reshape(nr, nr)
    counts = take(nr, np.uint32)
    id_ids, id_d = take(m * 32, np.uint32).reshape(m, 32), take(m * 32, np.float32).reshape(m, 32)
    full_ids, full_d = take(m * 32, np.uint32).reshape(m, 32), take(m * 32, np.float32).reshape(m, 32)
    nn1, d1 = take(m, np.uint32), take(m, np.float32)
    assert off == raw.size
    assert (rep < nr).all() and counts.sum() > 0
    X, Q = sample_inputs()
    own = [lists[j, :counts[j]] for j in range(nr)]
    allm = np.sort(np.concatenate(own))
    want_ids, want_d = _plan_oracle(oracle, X, Q, lambda i: own[rep[i]])
    np.testing.assert_array_equal(id_ids, want_ids)
    np.testing.assert_array_equal(id_d, want_d)
    want_ids, want_d = _plan_oracle(oracle, X, Q, lambda i: allm)
    np.testing.assert_array_equal(full_ids, want_ids)
    np.testing.assert_array_equal(full_d, want_d)
    np.testing.assert_array_equal(nn1, id_ids[:, 0])
    np.testing.assert_array_equal(d1, id_d[:, 0])


# ------------------------------------------------------------------ the double build
DOUBLE = ("-DRBC_REAL_DOUBLE",)


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference sources not present")
def test_reference_driver_double_build_links(engine_lib, tmp_path):
    """The reference's driver.cu compiled as its double build (real = double,
    defs.h:27-31) against include/ links against librbcgb_f64.so."""
    src = tmp_path / "driver.cu"
    src.write_bytes(open(REF_DRIVER, "rb").read())
    compile_program(str(src), str(tmp_path / "testRBC64"), engine_lib, extra=DOUBLE, lib="rbcgb_f64")


def test_double_library_exports_the_legacy_api(engine_lib):
    lib64 = os.path.join(os.path.dirname(engine_lib.LIB_PATH), "librbcgb_f64.so")
    out = subprocess.run(["nm", "-D", "--defined-only", lib64], capture_output=True, text=True, check=True).stdout
    for sym in ("_Z8buildRBC6matrixP9rbcStructjj", "_Z9kqueryRBC6matrix9rbcStruct9intMatrixS_",
                "_Z6bruteK6matrixS_9intMatrixS_", "_Z8bruteCPU6matrixS_Pj", "rbc_query_f64"):
        assert sym in out, sym


@pytest.mark.gpu
def test_legacy_driver_double_build(engine_lib, rbc, tmp_path):
    exe = compile_program(os.path.join(ROOT, "tests", "legacy_driver.cu"), str(tmp_path / "legacy_driver64"),
                          engine_lib, extra=DOUBLE, lib="rbcgb_f64")
    g = load_golden("f64_cases")
    xf, qf = str(tmp_path / "x64.bin"), str(tmp_path / "q64.bin")
    g["sample_X"].tofile(xf)
    g["sample_Q"].tofile(qf)
    outs = [str(tmp_path / f) for f in ("rbc.bin", "brute.bin", "nn1.bin")]
    r = subprocess.run([exe, xf, qf, "1024", "128", "16", "128"] + outs, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "one-shot list entries: 0" in r.stdout  # the one-shot lists are float-only
    for path in outs[:2]:
        raw = np.fromfile(path, np.uint8)
        ids = raw[: 128 * 32 * 4].view(np.uint32).reshape(128, 32)
        dists = raw[128 * 32 * 4:].view(np.float64).reshape(128, 32)
        np.testing.assert_array_equal(ids, g["sample_ids_l2"])
        np.testing.assert_array_equal(dists, g["sample_dists_l2"])
    raw = np.fromfile(outs[2], np.uint8)
    nn = raw[: 3 * 128 * 4].view(np.uint32)
    for j in range(3):
        np.testing.assert_array_equal(nn[j * 128:(j + 1) * 128], g["sample_ref_bruteCPU_1nn"])
    np.testing.assert_array_equal(raw[3 * 128 * 4:].view(np.float64), g["sample_dists_l2"][:, 0])
