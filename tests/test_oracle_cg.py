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


def test_bjac_factors_and_cg(orc):
    """The BJAC restatement: on every diagonal block of 32 rows the ILU(0)
    factors reproduce A on its pattern (L U = A there), the apply equals a
    dense solve with L U block by block, and CG with it reaches the direct
    solution in fewer iterations than with DIAG."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    from psfun_gb300 import matrices
    A = matrices.laplacian_2d(26)
    n, bs = A.shape[0], orc.BJAC_BLOCK_ROWS
    C = orc.Csr.from_scipy(A)
    P = orc.Bjac(C)
    f = P.factors()
    Ad = A.toarray()
    r = np.random.default_rng(2).standard_normal(n)
    z = P.apply(r)
    for b0 in range(0, n, bs):
        b1 = min(n, b0 + bs)
        m = b1 - b0
        L, U = np.eye(m), np.zeros((m, m))
        for i in range(b0, b1):
            for e in range(f["irp"][i], f["irp"][i + 1]):
                j = f["ja"][e]
                assert b0 <= j < b1
                (L if e < f["dpos"][i] else U)[i - b0, j - b0] = f["val"][e]
            assert f["udinv"][i] == 1.0 / U[i - b0, i - b0]
        blk = Ad[b0:b1, b0:b1]
        assert np.max(np.abs((L @ U - blk)[blk != 0])) <= 1e-13 * np.abs(blk).max()
        zz = np.linalg.solve(L @ U, r[b0:b1])
        assert np.linalg.norm(z[b0:b1] - zz) <= 1e-12 * np.linalg.norm(zz)
    b = np.random.default_rng(3).standard_normal(n)
    xs = spl.spsolve((A + 0.1 * sp.identity(n)).tocsc(), b)
    ob = orc.dcg(C, b, 1.0, 0.1, eps=1e-12, itmax=3000, istop=2, prec="BJAC")
    od = orc.dcg(C, b, 1.0, 0.1, eps=1e-12, itmax=3000, istop=2, prec="DIAG")
    assert np.linalg.norm(ob["x"] - xs) <= 1e-9 * np.linalg.norm(xs)
    assert ob["iter"] < od["iter"]
