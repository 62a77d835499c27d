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


def _index_file(n=64, d=4, nr=4, **hdr):
    """A small partition-only index file laid out as rbc_save writes one
    (persist.cu): 128-byte header, representative ids, representatives,
    list-major rows, partition arrays.  Keyword arguments override header
    fields; the arrays come back for editing."""
    import struct
    ld, dp = (d + 15) // 16 * 16, (d + 3) // 4 * 4
    per = n // nr
    h = dict(version=2, d=d, ld=ld, dp=dp, nr=nr, s=0, lds=0, kp=0, flags=1, ld64=0, metric=0, n=n, n_pad=0,
             xi_rows=0, min_list=per, max_list=per)
    h.update(hdr)
    arrays = {
        "rep_ids": np.arange(nr, dtype=np.uint32) * per,
        "R": np.zeros(((nr + 15) // 16 * 16, ld), np.float32),
        "Xp": np.zeros((n, ld), np.float32),
        "perm": np.arange(n, dtype=np.uint32),
        "offsets": np.arange(nr + 1, dtype=np.uint64) * per,
        "radius": np.ones(nr, np.float32),
        "owner": (np.arange(n) // max(per, 1)).astype(np.uint32),
    }
    return h, arrays


def _write_index(path, h, arrays, tail=b""):
    import struct
    head = b"RBCGB300" + struct.pack("<10Ii4x5Q32x", h["version"], h["d"], h["ld"], h["dp"], h["nr"], h["s"],
                                     h["lds"], h["kp"], h["flags"], h["ld64"], h["metric"], h["n"], h["n_pad"],
                                     h["xi_rows"], h["min_list"], h["max_list"])
    assert len(head) == 128
    body = b"".join(np.ascontiguousarray(arrays[k]).tobytes()
                    for k in ("rep_ids", "R", "Xp", "perm", "offsets", "radius", "owner"))
    path.write_bytes(head + body + tail)


def test_load_checks_every_field_before_the_device(engine_lib, tmp_path):
    """rbc_load refuses a damaged index file with RBC_ERR_IO before its first
    CUDA call: header fields, the file length, and the arrays that index into
    others (representative ids, list offsets, the partition's rows and
    owners, radii).  The intact file passes the checks (here, without a GPU,
    it then stops at the first CUDA call)."""
    import ctypes as C
    L = engine_lib.lib()
    p = tmp_path / "i.idx"

    def load(h, a, tail=b""):
        _write_index(p, h, a, tail)
        out = C.c_void_p()
        rc = L.rbc_load(str(p).encode(), C.byref(out))
        if rc == 0:
            L.rbc_destroy(out)
        return rc, L.rbc_last_error().decode()

    h, a = _index_file()
    rc, _ = load(h, a)
    assert rc in (0, engine_lib.ERR_CUDA), rc
    header_cases = [dict(d=600), dict(ld=32), dict(dp=8), dict(metric=5), dict(flags=1 | 0x40), dict(flags=0),
                    dict(flags=4 | 2, s=8, lds=16), dict(nr=65), dict(n=0), dict(min_list=3), dict(max_list=100),
                    dict(xi_rows=7), dict(flags=1 | 2, s=80, lds=80)]
    for case in header_cases:
        h2, a2 = _index_file(**case)
        rc, msg = load(h2, a2)
        assert rc == engine_lib.ERR_IO, (case, rc, msg)
    edits = [("offsets", 2, 10), ("offsets", 4, 63), ("offsets", 0, 1), ("perm", 5, 64), ("perm", 5, 6),
             ("owner", 3, 2), ("owner", 3, 9), ("radius", 1, np.nan), ("radius", 1, -1.0), ("rep_ids", 1, 0),
             ("rep_ids", 2, 64)]
    for name, i, v in edits:
        h2, a2 = _index_file()
        a2[name][i] = v
        rc, msg = load(h2, a2)
        assert rc == engine_lib.ERR_IO and "corrupt" in msg, (name, i, v, rc, msg)
    h2, a2 = _index_file()
    for tail in (b"\0" * 4,):
        rc, msg = load(h2, a2, tail)
        assert rc == engine_lib.ERR_IO and "longer" in msg, msg
    _write_index(p, h2, a2)
    p.write_bytes(p.read_bytes()[:-4])
    out = C.c_void_p()
    assert L.rbc_load(str(p).encode(), C.byref(out)) == engine_lib.ERR_IO
    assert b"truncated" in L.rbc_last_error()


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
