"""HHT rule (hhtmethod1) on the host and the quadrature-sum formula used by
the GPU path, checked with dense linear algebra on a small SPD matrix."""
import numpy as np
import pytest
import scipy.linalg as sl

from psfun_gb300 import matrices


def invsqrt(z):
    return 1.0 / np.sqrt(z)


def test_hht_product_equals_oracle(lib, orc):
    import psfun_gb300 as pg
    for N in (4, 10, 24):
        a = pg.hhtmethod1(invsqrt, N, [0.01, 4.0])
        b = orc.hhtmethod1(invsqrt, N, [0.01, 4.0])
        assert a[4] == 0 and b[4] == 0
        assert np.allclose(a[0], b[0], rtol=1e-14, atol=0)
        assert np.allclose(a[1], b[1], rtol=1e-13, atol=1e-300)
        assert abs(a[2] - b[2]) <= 1e-14 * abs(b[2]) and a[3] == b[3] == -1.0


def test_quadraturetest_scenario(orc):
    """quadraturetest.F90:60-68: sqrt(1+z), N = 10 on [0.01, 4] gives 10 finite poles/weights."""
    xi, c, eta, sign, info = orc.hhtmethod1(lambda z: np.sqrt(1.0 + z), 10, [0.01, 4.0])
    assert info == 0 and np.all(np.isfinite(xi)) and np.all(np.isfinite(c)) and sign == -1.0


@pytest.mark.parametrize("N,tol", [(8, 5e-3), (16, 1e-7), (24, 1e-11)])
def test_quadrature_sum_formula(orc, N, tol):
    """y = eta * A * Im(sum_j c_j (xi_j I - A)^{-1} x) approximates A^{-1/2} x."""
    A = matrices.laplacian_1d(12).toarray()
    w = np.linalg.eigvalsh(A)
    x = np.random.default_rng(0).standard_normal(12)
    xi, c, eta, sign, info = orc.hhtmethod1(invsqrt, N, [w[0], w[-1]])
    s = sum(cj * np.linalg.solve(xj * np.eye(12) + sign * A, x) for xj, cj in zip(xi, c))
    y = eta * A @ s.imag
    ref = sl.fractional_matrix_power(A, -0.5) @ x
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < tol
