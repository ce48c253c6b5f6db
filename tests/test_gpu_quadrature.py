"""Rational quadrature A^{-1/2} x (HHT rule, multi-shift solve sharing one
Lanczos basis) against exact spectral evaluation through the Kronecker
structure of the grid Laplacians, at test size and at the full 96^3 size."""
import numpy as np
import pytest

from oracle import exact
from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu


def apply_fun_3d(n1, x, fun):
    return exact.laplacian_3d_apply(n1, x, fun)


def run(n1, N, x, eps=1e-10):
    import psfun_gb300 as pg
    A = matrices.laplacian_3d(n1)
    q = pg.PsfunZQuadrature()
    info = q.computepoles(pg.hhtmethod1, lambda z: 1.0 / np.sqrt(z), N,
                          rparams=list(matrices.laplacian_3d_bounds(n1)))
    assert info == 0
    q.setmatrix(pg.CsrMatrix.from_scipy(A))
    return q, q.apply(x, eps=eps, itmax=3000)


@pytest.mark.parametrize("n1", [6, 16])
def test_quadrature_matches_its_rule(lib, n1):
    """Solver error alone: the GPU sum equals the same quadrature rule evaluated exactly."""
    x = np.random.default_rng(2).standard_normal(n1 ** 3)
    q, (y, info, it, err) = run(n1, 24, x)
    assert info == 0 and err < 1e-10
    def rule(L):
        s = sum(cj * 1.0 / (xj + q.sign * L) for xj, cj in zip(q.xi, q.c))
        return q.eta * L * np.imag(s)
    ref = apply_fun_3d(n1, x, rule)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-9


def test_laplace3d_96_full_size(lib):
    """A^{-1/2} x on the 96^3 Laplacian, N = 24.  Solver error: the GPU sum equals the HHT rule
    evaluated exactly in the eigenbasis.  The rule itself is only accurate to
    ~1.6e-6 at kappa ~ 3800 with 24 poles (a property of the published rule)."""
    p = matrices.laplace3d_invsqrt()
    q, (y, info, it, err) = run(96, 24, p.x, eps=1e-13)
    assert info == 0 and err < 1e-13

    def rule(L):
        s = sum(cj * 1.0 / (xj + q.sign * L) for xj, cj in zip(q.xi, q.c))
        return q.eta * L * np.imag(s)
    exact_rule = apply_fun_3d(96, p.x, rule)
    assert np.linalg.norm(y - exact_rule) / np.linalg.norm(exact_rule) < 1e-9
    ref = apply_fun_3d(96, p.x, lambda L: L ** -0.5)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 2e-6


def test_laplace3d_96_48_poles(lib):
    """The shifts share one Lanczos basis, so 48 poles cost the same Krylov steps:
    A^{-1/2} x on 96^3 to ~1e-12."""
    p = matrices.laplace3d_invsqrt()
    q, (y, info, it, err) = run(96, 48, p.x, eps=1e-13)
    assert info == 0
    ref = apply_fun_3d(96, p.x, lambda L: L ** -0.5)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-10


def test_zero_rhs(lib):
    _, (y, info, it, err) = run(6, 8, np.zeros(216))
    assert info == 0 and not np.any(y)
