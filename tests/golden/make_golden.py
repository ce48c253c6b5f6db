"""Generates the committed golden fixtures from a checkout of the reference's
sources (the fixtures travel with the tests; this script and the reference
checkout are needed only to regenerate them).

Usage: python tests/golden/make_golden.py <path to the psfun source tree>

1. utiltest_control.json -- the control values printed by the reference's own
   known-answer test, parsed as text from examples/utils/utiltest.f90:63-87.
2. laplacian50.json      -- a fingerprint of the reference's fixture matrix
   examples/polynomial/laplacian.mtx (checked equal to tridiag(1,-2,1), n=50).
3. driver_scenarios.npz  -- oracle outputs for the reference's driver
   scenarios on that matrix (arnolditest / lanczostest / serialtest with the
   driver's eps 1e-6, itmax 100, istop 1, x = ones) and for the
   100 x 100 5-point Laplacian problem (exp(-A)x, m <= 50, eps 1e-10).
"""
from __future__ import annotations

import hashlib
import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
REF = Path(".")  # set from the command line in main()


def utiltest_controls() -> dict:
    src = (REF / "examples/utils/utiltest.f90").read_text()
    out = {}
    m = re.search(r"should be (\d+)", src)
    out["horner_p1"] = float(m.group(1))
    m = re.search(r'"L = 0\.5 K = ([0-9.]+) Kp = ([0-9.]+) \(Control Values\)"', src)
    out["ellipkkp_L0.5"] = [float(m.group(1)), float(m.group(2))]
    m = re.search(r'"sn = ([0-9.]+) cn = ([0-9.]+) dn = ([0-9.]+) \(Control Values\)"', src)
    out["ellipj_u1_L0.5"] = [float(m.group(i)) for i in (1, 2, 3)]
    m = re.search(r'"sn = \(0\.0,([0-9.]+)\) cn = \(([0-9.]+),0\.0\) dn = \(([0-9.]+),0\.0\) \(Control Values\)"', src)
    out["ellipj_u0.5i_L1"] = {"sn": [0.0, float(m.group(1))], "cn": [float(m.group(2)), 0.0],
                              "dn": [float(m.group(3)), 0.0]}
    out["horner_coeffs"] = [132.0, 42.0, 14.0, 5.0, 2.0, 1.0, 0.0]
    out["source"] = "examples/utils/utiltest.f90:63-87"
    return out


def main():
    global REF
    if len(sys.argv) != 2 or not (Path(sys.argv[1]) / "examples/utils/utiltest.f90").is_file():
        raise SystemExit("usage: make_golden.py <psfun source tree (holding examples/utils/utiltest.f90)>")
    REF = Path(sys.argv[1])
    from oracle import oracle as orc
    from psfun_gb300 import matrices

    (HERE / "utiltest_control.json").write_text(json.dumps(utiltest_controls(), indent=1) + "\n")

    mtx = REF / "examples/polynomial/laplacian.mtx"
    A50 = matrices.read_matrix_market(mtx)
    T = -matrices.laplacian_1d(50)
    assert abs(A50 - T).max() == 0.0
    (HERE / "laplacian50.json").write_text(json.dumps({
        "source": "examples/polynomial/laplacian.mtx", "sha256": hashlib.sha256(mtx.read_bytes()).hexdigest(),
        "n": 50, "nnz_stored": 99, "equals": "tridiag(1,-2,1)"}, indent=1) + "\n")

    fix = {}
    A = orc.Csr.from_scipy(T)
    ones = np.ones(50)
    # arnolditest.F90:207-223 (EXP/GENPADE, driver overrides eps 1e-6, itmax 100, istop 1)
    r = orc.krylov("ARNOLDI", orc.serial("EXP", "GENPADE", 1.0), A, ones, 1e-6, itmax=100, istop=1)
    fix.update(arn_y=r["y"], arn_iter=r["iter"], arn_err=r["err"], arn_res=r["res"])
    # lanczostest with lanczos.inp's variant CHBSYM
    r = orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), A, ones, 1e-6, itmax=100, istop=1)
    fix.update(lz_y=r["y"], lz_iter=r["iter"], lz_err=r["err"], lz_res=r["res"])
    # serialtest.f90:86-114 with serial.inp (EXP/GENPADE, scaling 1, x = ones)
    y, info = orc.serial_apply(orc.serial("EXP", "GENPADE", 1.0), T.toarray(), ones)
    fix.update(serial_y=y)

    # 100x100 5-point Laplacian, exp(-A)x, m <= 50, eps 1e-10
    p = matrices.laplace2d_expm()
    C1 = orc.Csr.from_scipy(p.A)
    r = orc.krylov("ARNOLDI", orc.serial("EXP", "GENPADE", -1.0), C1, p.x, 1e-10, itmax=50, istop=1)
    fix.update(lap2d_arn_y=r["y"], lap2d_arn_iter=r["iter"], lap2d_arn_err=r["err"], lap2d_arn_res=r["res"])
    Cm = orc.Csr.from_scipy(-p.A)
    r = orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), Cm, p.x, 1e-10, itmax=50, istop=1)
    fix.update(lap2d_lz_y=r["y"], lap2d_lz_iter=r["iter"], lap2d_lz_err=r["err"], lap2d_lz_res=r["res"])
    # dense oracle: exp(-A) = exp(-T) (x) exp(-T) for the Kronecker sum
    X = p.x.reshape(100, 100)
    fix["lap2d_dense_y"] = orc.kron_expm_2d_times(matrices.laplacian_1d(100).toarray(), X).ravel()
    np.savez_compressed(HERE / "driver_scenarios.npz", **{k: np.asarray(v) for k, v in fix.items()})
    print({k: (v if np.ndim(v) == 0 else np.shape(v)) for k, v in fix.items()})


if __name__ == "__main__":
    main()
