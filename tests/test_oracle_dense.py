"""The dense f(H) restatements (DGPADM, CRAM, SASQ, TAYLOR, PHI, USERF/SYM)
against SciPy's expm on small matrices: pins the oracle where the reference
has no golden vectors."""
import numpy as np
import pytest
import scipy.linalg as sl


def _hess(m, seed, negdef=True):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((m, m))
    S = B @ B.T / m + np.eye(m)
    return -S if negdef else S


@pytest.mark.parametrize("m", [1, 2, 7, 20, 45])
@pytest.mark.parametrize("t", [1.0, -0.3, 2.5])
def test_dgpadm_matches_expm(orc, m, t):
    H = np.random.default_rng(m).standard_normal((m, m))
    E, info, ns = orc.dgpadm(H, t)
    assert info == 0
    ref = sl.expm(t * H)
    assert np.linalg.norm(E - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("variant", ["GENPADE", "CHBHES", "CHBSYM", "CHBGEN", "SASQ", "TAYLOR"])
def test_serial_exp_variants(orc, variant):
    m = 24
    H = _hess(m, 3)  # negative definite: CRAM is accurate there
    if variant == "CHBHES":
        H = np.triu(H, -1)  # upper Hessenberg
    x = np.random.default_rng(5).standard_normal(m)
    y, info = orc.serial_apply(orc.serial("EXP", variant, 0.7), H, x)
    assert info == 0
    ref = sl.expm(0.7 * H) @ x
    tol = 5e-13 if variant not in ("CHBHES", "CHBSYM", "CHBGEN") else 1e-11  # CRAM(14,14) partial fractions
    assert np.linalg.norm(y - ref) <= tol * np.linalg.norm(ref)


def test_default_variant_is_an_error(orc):
    """fname 'EXP' with the default variant 'EXPOKIT' errors (psfun_d_serial_mod.F90:387-390)."""
    y, info = orc.serial_apply(orc.serial("EXP", "EXPOKIT"), np.eye(3), np.ones(3))
    assert info == 4010


def test_names_are_case_sensitive(orc):
    y, info = orc.serial_apply(orc.serial("exp", "GENPADE"), np.eye(3), np.ones(3))
    assert info == 4010


@pytest.mark.parametrize("k", [1, 2, 3])
def test_phi_augmented(orc, k):
    m = 15
    H = _hess(m, 7)
    x = np.random.default_rng(9).standard_normal(m)
    y, info = orc.serial_apply(orc.serial("PHI", "", 0.5, phiorder=k), H, x)
    assert info == 0
    # phi_k(z) = sum_j z^j / (j+k)! through the eigendecomposition of the symmetric H
    w, V = np.linalg.eigh(0.5 * H)
    from math import factorial
    def phik(z):
        if abs(z) < 1e-3:
            return sum(z ** j / factorial(j + k) for j in range(12))
        s = np.exp(z) - sum(z ** j / factorial(j) for j in range(k))
        return s / z ** k
    ref = V @ (np.array([phik(z) for z in w]) * (V.T @ x))
    assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)


def test_userf_sym(orc):
    m = 12
    H = _hess(m, 11)
    x = np.ones(m)
    f = lambda v, k: np.exp(v)
    y, info = orc.serial_apply(orc.serial("USERF", "SYM", 1.3, f=f), H, x)
    assert info == 0
    ref = sl.expm(1.3 * H) @ x
    assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)


def test_serial_driver_scenario(orc):
    """serialtest.f90:86-114 (exp(A) 1 on laplacian.mtx) against expm and the fixture."""
    from pathlib import Path
    from psfun_gb300 import matrices
    T = (-matrices.laplacian_1d(50)).toarray()
    y, info = orc.serial_apply(orc.serial("EXP", "GENPADE", 1.0), T, np.ones(50))
    assert info == 0
    ref = sl.expm(T) @ np.ones(50)
    assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)
    fix = np.load(Path(__file__).parent / "golden" / "driver_scenarios.npz")
    assert np.linalg.norm(y - fix["serial_y"]) <= 1e-14 * np.linalg.norm(ref)
