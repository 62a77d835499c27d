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


def compile_program(src, out, engine_lib, extra=()):
    libdir = os.path.dirname(engine_lib.LIB_PATH)
    cmd = ["nvcc", "-O2", "-std=c++17", *extra, f"-I{INCLUDE}", src, "-o", out, f"-L{libdir}", "-lrbcgb",
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
