"""Shifted CG restatement (psfun_dcg.F90) against a sparse direct solve."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from psfun_gb300 import matrices


@pytest.mark.parametrize("prec", ["NONE", "DIAG"])
@pytest.mark.parametrize("istop", [1, 2])
def test_cg_shifted(orc, prec, istop):
    A = matrices.laplacian_2d(30)
    b = np.random.default_rng(2).standard_normal(A.shape[0])
    eta, zeta = 1.5, 0.3
    r = orc.dcg(orc.Csr.from_scipy(A), b, eta, zeta, eps=1e-12, itmax=2000, istop=istop, prec=prec)
    assert r["info"] == 0 and r["iter"] < 2000
    ref = spl.spsolve((eta * A + zeta * sp.identity(A.shape[0])).tocsc(), b)
    assert np.linalg.norm(r["x"] - ref) / np.linalg.norm(ref) < 1e-9


def test_cg_shiftedtest_scenario(orc):
    """shifted.inp: (-A + I) x = 1 with A = laplacian.mtx, DIAG, ISTOPC 2, eps 1e-7."""
    T = -matrices.laplacian_1d(50)
    r = orc.dcg(orc.Csr.from_scipy(T), np.ones(50), -1.0, 1.0, eps=1e-7, itmax=500, istop=2, prec="DIAG")
    assert r["info"] == 0 and r["err"] <= 1e-7
    M = (-T + sp.identity(50)).toarray()
    assert np.linalg.norm(M @ r["x"] - 1.0) <= 1e-7 * np.sqrt(50) * 1.0001


def test_cg_itmax_stops(orc):
    A = matrices.laplacian_2d(30)
    b = np.ones(A.shape[0])
    r = orc.dcg(orc.Csr.from_scipy(A), b, 1.0, 0.0, eps=1e-30, itmax=7, istop=2)
    assert r["iter"] == 7


@pytest.mark.parametrize("prec", ["NONE", "DIAG"])
def test_cg_cond_matches_dense_operator(orc, prec):
    """cond (psfun_dcg.F90:312-347): eig_max/eig_min of the CG tridiagonal.
    Run to convergence on a small SPD system, its extreme Ritz values are the
    extreme eigenvalues of the preconditioned operator D^{1/2}(eta A + zeta I)D^{1/2}."""
    A = matrices.laplacian_2d(12)
    b = np.random.default_rng(0).standard_normal(A.shape[0])
    r = orc.dcg_cond(orc.Csr.from_scipy(A), b, 1.0, 0.5, eps=1e-12, itmax=500, istop=2, prec=prec)
    assert r["info"] == 0 and len(r["td"]) == r["iter"]
    Ad = A.toarray()
    M = Ad + 0.5 * np.eye(A.shape[0])
    d = 1.0 / np.sqrt(np.diag(Ad)) if prec == "DIAG" else np.ones(A.shape[0])
    ev = np.linalg.eigvalsh(d[:, None] * M * d[None, :])
    assert r["cond"] == pytest.approx(ev[-1] / ev[0], rel=1e-10)
    # the per-iteration stopping values end at the returned err
    assert r["errh"][-1] == r["err"] and np.all(np.diff(np.log(r["errh"])) < 2.0)
