"""The testRBC command-line driver (the reference driver's interface,
driver.cu:22-198) and index files (rbc_save / rbc_load)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, load_golden


def cli(engine_lib):
    import build_ext
    return build_ext.build_cli()


def test_cli_usage_and_argument_errors(engine_lib):
    exe = cli(engine_lib)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and "usage" in r.stdout and "numReps" in r.stdout
    r = subprocess.run([exe, "-x", "a", "-q", "b", "-n", "100", "-m", "10", "-d", "4", "-r", "8"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "at least 32" in r.stderr
    r = subprocess.run([exe, "-x", "a", "-q", "b", "-n", "10", "-m", "10", "-d", "4", "-r", "40"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "more representatives than points" in r.stderr
    r = subprocess.run([exe, "-Z"], capture_output=True, text=True)
    assert r.returncode == 1 and "unrecognized option" in r.stderr
    r = subprocess.run([exe, "-D", "-M", "oneshot", "-x", "a", "-q", "b", "-n", "100", "-m", "10", "-d", "4", "-r",
                        "32"], capture_output=True, text=True)
    assert r.returncode == 1 and "double precision" in r.stderr
    r = subprocess.run([exe, "-x", "a", "-q", "b", "-n", "100", "-m", "10", "-d", "4", "-r", "32", "-k", "129"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "k must be in [1, 128]" in r.stderr


def test_load_rejects_bad_files(engine_lib, tmp_path):
    import ctypes as C
    L = engine_lib.lib()
    h = C.c_void_p()
    p = tmp_path / "bad.idx"
    p.write_bytes(b"NOTANIDX" + bytes(200))
    assert L.rbc_load(str(p).encode(), C.byref(h)) == engine_lib.ERR_IO
    assert L.rbc_load(str(tmp_path / "missing.idx").encode(), C.byref(h)) == engine_lib.ERR_IO


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["exact", "tc", "oneshot"])
def test_cli_on_sample_input(engine_lib, rbc, oracle, tmp_path, mode):
    exe = cli(engine_lib)
    out = str(tmp_path / "out.bin")
    idxf = str(tmp_path / "sample.idx")
    args = [exe, "-x", os.path.join(GOLDEN, "sample_db.bin"), "-q", os.path.join(GOLDEN, "sample_queries.bin"),
            "-n", "1024", "-m", "128", "-d", "16", "-r", "128", "-o", out, "-M", mode, "-S", idxf, "-e"]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, np.uint8)
    ids = raw[: 128 * 32 * 4].view(np.uint32).reshape(128, 32)
    dists = raw[128 * 32 * 4:].view(np.float32).reshape(128, 32)
    g = load_golden("sample_input")
    if mode == "oneshot":
        X = np.fromfile(os.path.join(GOLDEN, "sample_db.bin"), np.float32).reshape(1024, 16)
        Q = np.fromfile(os.path.join(GOLDEN, "sample_queries.bin"), np.float32).reshape(128, 16)
        idx = rbc.Index.load(idxf)
        reps = idx.reps()
        lists, counts, _ = oracle.oneshot_build(X, reps, 128)
        oi, od = oracle.oneshot_query(X, reps, lists, counts, Q, 32)
        np.testing.assert_array_equal(ids, oi)
        np.testing.assert_array_equal(dists, od)
        idx.close()
    else:
        np.testing.assert_array_equal(ids, g["ids_l2"])
        np.testing.assert_array_equal(dists, g["dists_l2"])
        assert "avg overlap = 32.0000/32" in r.stdout
    # the saved index answers the same from a new process
    out2 = str(tmp_path / "out2.bin")
    r = subprocess.run(args[:args.index("-r")] + ["-L", idxf, "-o", out2, "-M", mode], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert open(out, "rb").read() == open(out2, "rb").read()


@pytest.mark.gpu
def test_index_file_round_trip(rbc, tmp_path):
    X = rbc.synth(1, 4, 0, 30000, 64, ncomp=50, sigma_lo=0.05, sigma_hi=0.05)
    Q = rbc.synth(1, 4, 1, 500, 64, ncomp=50, sigma_lo=0.05, sigma_hi=0.05)
    idx = rbc.Index(X, 200, s=150, seed=9, flags=rbc.BUILD_PARTITION | rbc.BUILD_ONESHOT | rbc.BUILD_BF16)
    path = str(tmp_path / "x.idx")
    idx.save(path)
    back = rbc.Index.load(path)
    assert back.info() == idx.info()
    np.testing.assert_array_equal(back.reps(), idx.reps())
    for a, b in zip(back.partition(), idx.partition()):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(back.oneshot(), idx.oneshot()):
        np.testing.assert_array_equal(a, b)
    for mode in (rbc.QUERY_EXACT, rbc.QUERY_EXACT_TC, rbc.QUERY_ONESHOT):
        i1, d1 = idx.query(Q, 10, mode=mode)
        i2, d2 = back.query(Q, 10, mode=mode)
        assert (i1 == i2).all() and (d1 == d2).all()
    with open(path, "r+b") as f:  # a truncated file is an error, not a crash
        f.truncate(os.path.getsize(path) // 2)
    with pytest.raises(rbc.RBCError) as e:
        rbc.Index.load(path)
    assert e.value.code == rbc.ERR_IO
    idx.close()
    back.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["exact", "tc"])
def test_cli_double_build(engine_lib, rbc, tmp_path, mode):
    """-D: the reference's real = double build: 8-byte values in and out."""
    exe = cli(engine_lib)
    g = load_golden("f64_cases")
    xf, qf, out = str(tmp_path / "x64.bin"), str(tmp_path / "q64.bin"), str(tmp_path / "out64.bin")
    g["sample_X"].astype(np.float64).tofile(xf)
    g["sample_Q"].astype(np.float64).tofile(qf)
    idxf = str(tmp_path / "x64.idx")
    args = [exe, "-D", "-x", xf, "-q", qf, "-n", "1024", "-m", "128", "-d", "16", "-r", "128", "-o", out, "-M", mode,
            "-S", idxf, "-e"]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, np.uint8)
    assert raw.size == 128 * 32 * (4 + 8)
    ids = raw[: 128 * 32 * 4].view(np.uint32).reshape(128, 32)
    dists = raw[128 * 32 * 4:].view(np.float64).reshape(128, 32)
    np.testing.assert_array_equal(ids, g["sample_ids_l2"])
    np.testing.assert_array_equal(dists, g["sample_dists_l2"])
    assert "avg overlap = 32.0000/32" in r.stdout
    out2 = str(tmp_path / "out64b.bin")
    r = subprocess.run(args[:args.index("-r")] + ["-L", idxf, "-o", out2, "-M", mode], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert open(out, "rb").read() == open(out2, "rb").read()
    # an index of one precision is refused by the other
    r = subprocess.run([a for a in args[:args.index("-r")] if a != "-D"] + ["-L", idxf], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "other precision" in r.stderr
