"""The dense solve of the Pade step (dense.cuh::cta_lu_solve) on the device:
A X = B with partial pivoting, on one block and on a group of 8 blocks,
orders 1..150 (both sides of the one-barrier factorisation's limit, 128), on
random matrices, on matrices whose every step exchanges rows, and on an
exactly singular one.  The normwise backward error must stay at rounding
level, the pivot rows must be IDAMAX's (the first row of largest magnitude,
as a host elimination chooses them), and a zero pivot must be reported.

The Pade denominator that DGPADM solves after its scaling is diagonally
dominant and never pivots, so the public entries cannot reach the pivoting
cases: the check is a small CUDA program (tests/cuda/dense_lu_check.cu)
compiled against the library's device headers."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_dense_lu_solve_device(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "dense_lu_check"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(ROOT / "psfun_gb300" / "csrc"),
                    "-o", str(exe), str(ROOT / "tests" / "cuda" / "dense_lu_check.cu")], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    cases = []
    for line in out.stdout.splitlines():
        t = line.split()
        assert t[0] == "case", line
        d = dict(zip(t[0::2], t[1::2]))
        cases.append((d["case"], int(d["m"]), int(d["G"]), int(d["ok"]), float(d["berr"]), int(d["pivdiff"]),
                      int(d["grouperr"])))
    assert len(cases) == 13 * 2 * 2 + 10 * 2
    for name, m, G, ok, berr, pivdiff, grouperr in cases:
        assert grouperr == 0, (name, m, G)
        if name == "singular":
            assert ok == 0, (name, m, G)
        else:
            assert ok == 1, (name, m, G)
            assert berr <= 1e-13, (name, m, G, berr)
            assert pivdiff == 0, (name, m, G, pivdiff)
