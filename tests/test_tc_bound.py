"""Soundness of the tensor form's certificate, checked on the CPU.

tests/tc_bound_check.cu restates on the host the quantities the tensor-core
list search derives for a (query, row) pair (centered half-precision
operands, w and its BF16 pieces, the query norm, the list bounds, Dqr) and
the tensor-core value under four models of the FP32 accumulation, then checks
|approx - exact| <= tc_error_bound (csrc/tc.cuh) for every pair, exact being
the reference's sequential FP32 distance (utils.cu:183-191).  The bound is
doubled as a margin, so the error must also stay within half of it.
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "tc_bound_check.cu")
CSRC = os.path.join(ROOT, "randomballcover-gpu_gb300", "csrc")


@pytest.fixture(scope="module")
def bound_check(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path_factory.mktemp("tcb") / "tc_bound_check")
    # host code only; no contraction of the restated roundings into FMAs
    subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
                    "-Xcompiler", "-ffp-contract=off", SRC, "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2])
def test_certificate_covers_every_pair(bound_check, seed):
    r = subprocess.run([bound_check, str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = [ln for ln in r.stdout.splitlines() if " pairs " in ln]
    assert len(rows) == 8, r.stdout
    for ln in rows:
        name = ln.split()[0]
        pairs = int(re.search(r"pairs (\d+)", ln).group(1))
        assert pairs > 0 and " violations 0 " in ln, ln
        worst = [float(v) for v in re.findall(r"=([0-9.eE+-]+)", ln)]
        assert len(worst) == 4, ln
        assert max(worst) <= 0.5, f"{name}: error above the undoubled bound: {ln}"
    # inexact operands and large cancelling sums do produce rounding error:
    # the check is not vacuous
    assert any(float(v) > 0 for v in re.findall(r"fractional_queries\S* .*?rz_step=([0-9.eE+-]+)", r.stdout))
    assert "total violations 0" in r.stdout


def test_underestimating_bound_is_caught(bound_check):
    """A bound planted 64 times too small (the checker's own factor) must
    fail: the check sees the rounding errors it is meant to cover."""
    r = subprocess.run([bound_check, "1", "0.015625"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 1, r.stdout + r.stderr
    assert "violation bf16_fractional_queries" in r.stdout or "violations 0 " not in r.stdout
    assert int(re.search(r"total violations (\d+)", r.stdout).group(1)) > 0
