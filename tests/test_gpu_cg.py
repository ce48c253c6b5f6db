"""Shifted CG (psb_krylov -> psfun_dcg_vect) on the GPU against the oracle."""
import numpy as np
import pytest
import scipy.sparse as sp

from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["NONE", "DIAG", "BJAC"])
@pytest.mark.parametrize("istop", [1, 2])
def test_cg_vs_oracle(lib, orc, prec, istop):
    import psfun_gb300 as pg
    A = matrices.laplacian_2d(40)
    b = np.random.default_rng(2).standard_normal(A.shape[0])
    eta, zeta = 1.5, 0.3
    x, info, it, err = pg.psb_krylov("CG", pg.CsrMatrix.from_scipy(A), prec, b, eta, zeta, np.zeros_like(b),
                                     1e-12, itmax=3000, istop=istop)
    o = orc.dcg(orc.Csr.from_scipy(A), b, eta, zeta, eps=1e-12, itmax=3000, istop=istop, prec=prec)
    assert info == 0 and o["info"] == 0
    assert abs(it - o["iter"]) <= 1
    assert np.linalg.norm(x - o["x"]) <= 1e-9 * np.linalg.norm(o["x"])
    assert err <= 1e-12


def test_shiftedtest_scenario(lib):
    import psfun_gb300 as pg
    T = -matrices.laplacian_1d(50)
    x, info, it, err = pg.psb_krylov("CG", pg.CsrMatrix.from_scipy(T), "DIAG", np.ones(50), -1.0, 1.0,
                                     np.zeros(50), 1e-7, itmax=500, istop=2)
    assert info == 0 and err <= 1e-7
    M = (-T + sp.identity(50)).toarray()
    assert np.linalg.norm(M @ x - 1.0) <= 1e-7 * np.sqrt(50) * 1.0001


def test_cg_itmax_and_unknown_method(lib, orc):
    import psfun_gb300 as pg
    A = matrices.laplacian_2d(30)
    b = np.ones(A.shape[0])
    x, info, it, err = pg.psb_krylov("BICGSTAB", pg.CsrMatrix.from_scipy(A), "NONE", b, 1.0, 0.0,
                                     np.zeros_like(b), 1e-30, itmax=7, istop=2)
    o = orc.dcg(orc.Csr.from_scipy(A), b, 1.0, 0.0, eps=1e-30, itmax=7, istop=2)
    assert info == 0 and it == o["iter"] == 7
    assert np.linalg.norm(x - o["x"]) <= 1e-12 * np.linalg.norm(o["x"])


def test_cg_errors(lib):
    import psfun_gb300 as pg
    a = pg.CsrMatrix.from_scipy(matrices.laplacian_2d(8))
    b = np.ones(64)
    assert pg.psb_krylov("CG", a, "NONE", b, 1.0, 0.0, np.zeros(64), 1e-8, istop=3)[1] == 5001
    assert pg.psb_krylov("CG", a, "ILU99", b, 1.0, 0.0, np.zeros(64), 1e-8)[1] == 111


@pytest.mark.parametrize("prec", ["NONE", "DIAG", "BJAC"])
def test_cg_cond_vs_oracle(lib, orc, prec):
    """The optional cond: the GPU's CG tridiagonal eigenvalue ratio against the
    oracle's (LAPACK's tridiagonal solver on the oracle's alphas and betas)."""
    import psfun_gb300 as pg
    A = matrices.laplacian_2d(40)
    b = np.random.default_rng(5).standard_normal(A.shape[0])
    x, info, it, err, cond = pg.psb_krylov("CG", pg.CsrMatrix.from_scipy(A), prec, b, 1.0, 0.25,
                                           np.zeros_like(b), 1e-11, itmax=3000, istop=2, cond=True)
    o = orc.dcg_cond(orc.Csr.from_scipy(A), b, 1.0, 0.25, eps=1e-11, itmax=3000, istop=2, prec=prec)
    assert info == 0 and abs(it - o["iter"]) <= 1
    assert cond == pytest.approx(o["cond"], rel=1e-8)
    # without cond the solution is the same
    x2, info2, it2, err2 = pg.psb_krylov("CG", pg.CsrMatrix.from_scipy(A), prec, b, 1.0, 0.25, np.zeros_like(b),
                                         1e-11, itmax=3000, istop=2)
    assert np.array_equal(x, x2) and it == it2


def test_cg_itrace_log(lib, capfd):
    import psfun_gb300 as pg
    A = matrices.laplacian_2d(30)
    b = np.ones(A.shape[0])
    capfd.readouterr()
    x, info, it, err = pg.psb_krylov("CG", pg.CsrMatrix.from_scipy(A), "DIAG", b, 1.0, 0.5, np.zeros_like(b), 1e-10,
                                     itmax=500, istop=2, itrace=4)
    lines = [l for l in capfd.readouterr().out.splitlines() if l.startswith("CG:")]
    assert info == 0
    its = [int(l.split()[1]) for l in lines[1:-1]]
    assert its == list(range(4, it + 1, 4))
    assert f"converged after {it} iterations" in lines[-1]


@pytest.mark.parametrize("A_name", ["laplace3d_48", "rgg_20000", "unsorted_dup", "tail_block"])
def test_cg_bjac_vs_oracle(lib, orc, A_name):
    """BJAC (block Jacobi, ILU(0) on the diagonal blocks of 32 rows) against
    the oracle's restatement: a 3-D Laplacian whose blocks cross the row
    ranges of the persistent kernel's blocks (tiles of up to 480 rows), a kNN
    graph Laplacian (irregular rows), a matrix stored with unsorted rows and a
    duplicated entry, and a size that leaves a short last block.  On the
    grid-ordered Laplacians BJAC needs fewer iterations than DIAG."""
    import psfun_gb300 as pg
    if A_name == "laplace3d_48":
        A = matrices.laplacian_3d(48)
    elif A_name == "rgg_20000":
        A = matrices.rgg_knn_laplacian(20000, 8, np.random.default_rng(7))
    elif A_name == "tail_block":
        A = matrices.laplacian_2d(37, 29)
    else:
        A = matrices.laplacian_2d(30).tocsr()
    n = A.shape[0]
    b = np.random.default_rng(9).standard_normal(n)
    if A_name == "unsorted_dup":
        irp, ja, val = A.indptr.copy(), A.indices.copy(), A.data.copy()
        for i in range(n):  # reverse every row, then split the diagonal of row 5 into two entries
            s_, e_ = irp[i], irp[i + 1]
            ja[s_:e_], val[s_:e_] = ja[s_:e_][::-1].copy(), val[s_:e_][::-1].copy()
        k = irp[5] + list(ja[irp[5]:irp[6]]).index(5)
        ja = np.insert(ja, k + 1, 5)
        half = val[k] / 2
        val[k] = half
        val = np.insert(val, k + 1, half)
        irp[6:] += 1
        a = pg.CsrMatrix(irp, ja, val)
        oa = orc.Csr(irp, ja, val)
    else:
        a = pg.CsrMatrix.from_scipy(A)
        oa = orc.Csr.from_scipy(A)
    x, info, it, err = pg.psb_krylov("CG", a, "BJAC", b, 1.0, 0.05, np.zeros(n), 1e-11, itmax=5000, istop=2)
    o = orc.dcg(oa, b, 1.0, 0.05, eps=1e-11, itmax=5000, istop=2, prec="BJAC")
    d = orc.dcg(oa, b, 1.0, 0.05, eps=1e-11, itmax=5000, istop=2, prec="DIAG")
    assert info == 0 and o["info"] == 0
    assert abs(it - o["iter"]) <= 1, (it, o["iter"])
    assert np.linalg.norm(x - o["x"]) <= 1e-9 * np.linalg.norm(o["x"])
    if A_name != "rgg_20000":  # a random graph ordering leaves weakly coupled rows in each block
        assert it < d["iter"], (it, d["iter"])
