"""Pins the oracle and the product's host-side elliptic/Horner routines to the
reference's only known-answer values (examples/utils/utiltest.f90:63-87)."""
import json
from pathlib import Path

import numpy as np
import pytest

CTRL = json.loads((Path(__file__).parent / "golden" / "utiltest_control.json").read_text())
TOL = 5e-15  # the control values are printed with 15 decimals


def test_oracle_horner(orc):
    assert orc.horner(CTRL["horner_coeffs"], 1.0) == CTRL["horner_p1"]


def test_oracle_ellipkkp(orc):
    K = orc.ellipkkp(0.5)
    assert np.allclose(K, CTRL["ellipkkp_L0.5"], rtol=0, atol=TOL)


def test_oracle_real_ellipj(orc):
    assert np.allclose(orc.d_ellipj(1.0, 0.5), CTRL["ellipj_u1_L0.5"], rtol=0, atol=TOL)


def test_oracle_complex_ellipj(orc):
    sn, cn, dn = orc.z_ellipj(0.5j, 1.0)
    c = CTRL["ellipj_u0.5i_L1"]
    for got, want in ((sn, c["sn"]), (cn, c["cn"]), (dn, c["dn"])):
        assert abs(got - complex(*want)) <= TOL


def test_product_host_routines_match_controls(lib):
    import psfun_gb300 as pg
    assert pg.horner(CTRL["horner_coeffs"], 1.0) == CTRL["horner_p1"]
    assert np.allclose(pg.ellipkkp(0.5), CTRL["ellipkkp_L0.5"], rtol=0, atol=TOL)
    assert np.allclose(pg.ellipj(1.0, 0.5), CTRL["ellipj_u1_L0.5"], rtol=0, atol=TOL)
    sn, cn, dn = pg.ellipj(0.5j, 1.0)
    c = CTRL["ellipj_u0.5i_L1"]
    for got, want in ((sn, c["sn"]), (cn, c["cn"]), (dn, c["dn"])):
        assert abs(got - complex(*want)) <= TOL


@pytest.mark.parametrize("L", [0.05, 0.3, 1.0, 3.0, 9.9, 10.5])
def test_product_elliptic_equals_oracle(lib, orc, L):
    import psfun_gb300 as pg
    assert np.array_equal(pg.ellipkkp(L), orc.ellipkkp(L))
    for u in (0.1, 0.7, 1.3):
        assert np.allclose(pg.ellipj(u, L), orc.d_ellipj(u, L), rtol=1e-15, atol=1e-15)
    K = orc.ellipkkp(L)
    for u in (0.3 + 0.2j, -0.4 + 0.5 * K[1] * 1j, 0.9 + 0.1j):
        a = pg.ellipj(complex(u), L)
        b = orc.z_ellipj(complex(u), L)
        for x, y in zip(a, b):
            assert abs(x - y) <= 1e-13 * max(1.0, abs(y))


def test_fixture_matrix_fingerprint():
    """The reference's fixture (laplacian.mtx) is tridiag(1,-2,1), n = 50."""
    fp = json.loads((Path(__file__).parent / "golden" / "laplacian50.json").read_text())
    from psfun_gb300 import matrices
    T = -matrices.laplacian_1d(50)
    assert fp["n"] == 50 and fp["equals"] == "tridiag(1,-2,1)"
    assert T.nnz == 2 * fp["nnz_stored"] - 50


@pytest.mark.parametrize("L", [0.02, 0.05, 0.3, 1.0, 3.0, 9.9, 10.5])
def test_product_elliptic_equals_scipy(lib, L):
    """An independent pin: K and K' (ellipkkp, m = exp(-2 pi L)) against SciPy's
    ellipk / ellipkm1, real sn/cn/dn against scipy.special.ellipj, and, for
    moderate L, purely imaginary arguments through Jacobi's imaginary
    transformation sn(iy|m) = i sc(y|1-m), cn(iy|m) = nc(y|1-m),
    dn(iy|m) = dc(y|1-m)."""
    ss = pytest.importorskip("scipy.special")
    import psfun_gb300 as pg
    m = np.exp(-2.0 * np.pi * L)
    K, Kp = pg.ellipkkp(L)
    assert abs(K / ss.ellipk(m) - 1.0) <= 4e-16
    assert abs(Kp / ss.ellipkm1(m) - 1.0) <= 4e-16
    for u in (0.1, 0.7, 1.3, 2.9):
        got = np.array(pg.ellipj(u, L))
        want = np.array(ss.ellipj(u, m)[:3])
        assert np.abs(got - want).max() <= 2e-15
    if L <= 1.0:
        for y in (0.2, 0.6):
            sn, cn, dn = pg.ellipj(complex(0.0, y), L)
            s1, c1, d1, _ = ss.ellipj(y, 1.0 - m)
            for got, want in ((sn, 1j * s1 / c1), (cn, 1.0 / c1), (dn, d1 / c1)):
                assert abs(got - want) <= 1e-14 * max(1.0, abs(want))
