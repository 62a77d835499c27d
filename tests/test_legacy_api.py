"""The reference's C++ API as a drop-in: programs written for it compile
against include/ and link against librbcgb.so; on the GPU they return the
oracle's neighbours."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, load_golden

INCLUDE = os.path.join(ROOT, "include")
REF_DRIVER = "/root/reference/driver.cu"


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
