"""The C-ABI library without a GPU: it builds, loads, exports every declared
symbol, and its host-only paths (file formats, argument checks) behave."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, sample_inputs

INCLUDE = os.path.join(ROOT, "include")


def declared(header):
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    names = re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", src, flags=re.M)
    return [n for n in names if n not in ("if", "while", "return", "sizeof")]


def exported(lib_path):
    out = subprocess.run(["nm", "-D", "-C", "--defined-only", lib_path], capture_output=True, text=True,
                         check=True).stdout
    names = set()
    for line in out.splitlines():
        parts = line.split(None, 2)
        if len(parts) == 3 and parts[1] in ("T", "W"):
            names.add(parts[2].split("(")[0])
    return names


def test_every_declared_symbol_is_exported(engine_lib):
    have = exported(engine_lib.LIB_PATH)
    missing = []
    for h in ("rbc_gb300.h", "rbc.h", "brute.h", "utils.h", "utilsGPU.h"):
        names = declared(h)
        assert names, h
        missing += [f"{h}:{n}" for n in names if n not in have]
    assert not missing, missing


def test_c_abi_signatures_cover_header(engine_lib):
    names = set(declared("rbc_gb300.h"))
    assert names == set(engine_lib.SIGNATURES), names ^ set(engine_lib.SIGNATURES)


def test_legacy_names_have_reference_mangling(engine_lib):
    """Programs built against the reference link to these C++ symbols."""
    out = subprocess.run(["nm", "-D", "--defined-only", engine_lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    for sym in ("_Z8buildRBC6matrixP9rbcStructjj", "_Z9kqueryRBC6matrix9rbcStruct9intMatrixS_",
                "_Z8queryRBC6matrix9rbcStructPjPf", "_Z10destroyRBCP9rbcStruct", "_Z6bruteK6matrixS_9intMatrixS_",
                "_Z8bruteCPU6matrixS_Pj", "_Z11bruteSearch6matrixS_Pj", "_Z15bruteRangeCount6matrixS_PfPj",
                "_Z7distVec6matrixS_jj", "_Z7initMatP6matrixjj",
                # the query plan of rbc.h:22-25
                "_Z12initCompPlanP8compPlan10charMatrixPjS2_j", "_Z12freeCompPlanP8compPlan",
                "_Z10computeNNs6matrix9intMatrixS_Pj8compPlanS1_Pfj",
                "_Z11computeKNNs6matrix9intMatrixS_Pj8compPlanS0_S_j"):
        assert sym in out, sym


def test_status_strings_and_argument_errors(engine_lib):
    L = engine_lib.lib()
    assert L.rbc_status_string(0) == b"ok"
    assert L.rbc_status_string(engine_lib.ERR_ITER_LIMIT) == b"bounded device wait ran out"
    h = C.c_void_p()
    assert L.rbc_build(None, 10, 4, 4, None, None, C.byref(h)) == engine_lib.ERR_INVALID
    assert b"params" in L.rbc_last_error()
    p = engine_lib.BuildParams(0, 0, 0, 0, 0, None)
    x = np.zeros((10, 4), np.float32)
    assert L.rbc_build(x.ctypes.data, 10, 4, 4, C.byref(p), None, C.byref(h)) == engine_lib.ERR_INVALID
    p.num_reps = 11
    assert L.rbc_build(x.ctypes.data, 10, 4, 4, C.byref(p), None, C.byref(h)) == engine_lib.ERR_INVALID
    p.num_reps = 2
    assert L.rbc_build(x.ctypes.data, 10, 4, 3, C.byref(p), None, C.byref(h)) == engine_lib.ERR_INVALID
    assert L.rbc_build(x.ctypes.data, 10, 600, 600, C.byref(p), None, C.byref(h)) == engine_lib.ERR_UNSUPPORTED
    p.metric = 7
    assert L.rbc_build(x.ctypes.data, 10, 4, 4, C.byref(p), None, C.byref(h)) == engine_lib.ERR_INVALID
    assert L.rbc_query(None, None, 1, 4, 1, 0, None, None, 1, None) == engine_lib.ERR_INVALID
    assert L.rbc_brute_knn(None, 1, 4, None, 1, 4, 4, 0, 0, None, None, 1, None) == engine_lib.ERR_INVALID
    assert L.rbc_brute_knn(None, 1, 4, None, 1, 4, 4, 129, 0, None, None, 129, None) == engine_lib.ERR_INVALID
    assert b"[1, 128]" in L.rbc_last_error()
    assert L.rbc_synth(9, 0, 0, 0, 1, 4, 4, None, 1, 0.0, 0.0, None) == engine_lib.ERR_INVALID
    assert L.rbc_destroy(None) == 0


def test_binary_format_round_trip(engine_lib, tmp_path):
    X, Q = sample_inputs()
    p = str(tmp_path / "db.bin")
    engine_lib.write_matrix_bin(p, X)
    assert open(p, "rb").read() == X.tobytes()  # headerless row-major float32
    back = engine_lib.read_matrix_bin(p, 1024, 16, ld=32)  # padded read, as readData does
    np.testing.assert_array_equal(back[:, :16], X)
    assert (back[:, 16:] == 0).all()
    with pytest.raises(engine_lib.RBCError) as e:
        engine_lib.read_matrix_bin(p, 1025, 16)  # short file
    assert e.value.code == engine_lib.ERR_IO
    with pytest.raises(engine_lib.RBCError):
        engine_lib.read_matrix_bin(str(tmp_path / "missing.bin"), 1, 1)


def test_text_format_reads_reference_style_text(engine_lib, tmp_path):
    X, _ = sample_inputs()
    p = str(tmp_path / "db.txt")
    with open(p, "w") as f:
        for row in X[:50]:
            f.write(" ".join("%.7e" % v for v in row) + "\n")
    back = engine_lib.read_matrix_text(p, 50, 16)
    np.testing.assert_array_equal(back, X[:50])


def test_neighbor_output_layout(engine_lib, tmp_path):
    ids = np.arange(6, dtype=np.uint32).reshape(2, 3)
    dists = np.arange(6, dtype=np.float32).reshape(2, 3) / 4
    p = str(tmp_path / "out.bin")
    engine_lib.write_neighbors_bin(p, ids, dists)
    raw = open(p, "rb").read()
    assert raw == ids.tobytes() + dists.tobytes()  # all ids, then all distances
    t = str(tmp_path / "out.txt")
    engine_lib.write_neighbors_text(t, ids, dists)
    lines = open(t).read().splitlines()
    assert lines[0] == "0 1 2 " and lines[2] == "0.000000 0.250000 0.500000 "
