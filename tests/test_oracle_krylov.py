"""The Arnoldi / Lanczos restatements: control flow and quirks of the
reference, accuracy against dense oracles, and regression against the
committed fixtures."""
from pathlib import Path

import numpy as np
import pytest

from psfun_gb300 import matrices

FIX = np.load(Path(__file__).parent / "golden" / "driver_scenarios.npz")


def test_laplace2d_100_arnoldi_vs_dense(orc):
    p = matrices.laplace2d_expm()
    r = orc.krylov("ARNOLDI", orc.serial("EXP", "GENPADE", -1.0), orc.Csr.from_scipy(p.A), p.x, 1e-10, itmax=50)
    assert r["info"] == 0 and r["iter"] == 18
    dense = FIX["lap2d_dense_y"]
    rel = np.linalg.norm(r["y"] - dense) / np.linalg.norm(dense)
    assert rel < 1e-10
    assert np.array_equal(r["y"], FIX["lap2d_arn_y"]) or np.linalg.norm(r["y"] - FIX["lap2d_arn_y"]) < 1e-13


def test_laplace2d_100_lanczos_vs_dense(orc):
    p = matrices.laplace2d_expm()
    r = orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), orc.Csr.from_scipy(-p.A), p.x, 1e-10, itmax=50)
    assert r["info"] == 0
    dense = FIX["lap2d_dense_y"]
    assert np.linalg.norm(r["y"] - dense) / np.linalg.norm(dense) < 1e-10


def test_drop_last_quirk(orc):
    """Assembly sums yk(1..itx-1) while yk has itx entries (psfun_d_arnoldi.f90:325-328):
    keeping every term is more accurate."""
    p = matrices.laplace2d_expm()
    A = orc.Csr.from_scipy(p.A)
    r1 = orc.krylov("ARNOLDI", orc.serial("EXP", "GENPADE", -1.0), A, p.x, 1e-10, itmax=50, drop_last=True)
    r2 = orc.krylov("ARNOLDI", orc.serial("EXP", "GENPADE", -1.0), A, p.x, 1e-10, itmax=50, drop_last=False)
    d = FIX["lap2d_dense_y"]
    e1 = np.linalg.norm(r1["y"] - d) / np.linalg.norm(d)
    e2 = np.linalg.norm(r2["y"] - d) / np.linalg.norm(d)
    assert e2 < e1


def test_driver_scenarios_regression(orc):
    T = orc.Csr.from_scipy(-matrices.laplacian_1d(50))
    r = orc.krylov("ARNOLDI", orc.serial("EXP", "GENPADE", 1.0), T, np.ones(50), 1e-6, itmax=100)
    assert r["iter"] == FIX["arn_iter"] and np.allclose(r["y"], FIX["arn_y"], rtol=1e-14, atol=0)
    r = orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), T, np.ones(50), 1e-6, itmax=100)
    assert r["iter"] == FIX["lz_iter"] and np.allclose(r["y"], FIX["lz_y"], rtol=1e-14, atol=0)


def test_istop_and_itmax_errors(orc):
    T = orc.Csr.from_scipy(-matrices.laplacian_1d(20))
    fun = orc.serial("EXP", "GENPADE", 1.0)
    assert orc.krylov("ARNOLDI", fun, T, np.ones(20), 1e-6, istop=3)["info"] == 5001
    assert orc.krylov("LANCZOS", fun, T, np.ones(20), 1e-6, istop=0)["info"] == 5001
    assert orc.krylov("ARNOLDI", fun, T, np.ones(20), 1e-6, itmax=1)["info"] == 4011
    bad = orc.serial("EXP", "EXPOKIT", 1.0)
    assert orc.krylov("ARNOLDI", bad, T, np.ones(20), 1e-6)["info"] == 4011


def test_istop2_runs_to_itmax(orc):
    """istop = 2 disables the estimate: the loop runs to nl and f is evaluated on
    H(1:nl-2,1:nl-2) (psfun_d_arnoldi.f90:282-314)."""
    A = matrices.laplacian_2d(20)
    x = matrices.unit(np.random.default_rng(1).standard_normal(400))
    r = orc.krylov("ARNOLDI", orc.serial("EXP", "GENPADE", -0.1), orc.Csr.from_scipy(A), x, 1e-10, itmax=30,
                   istop=2)
    assert r["info"] == 0 and r["iter"] == 29 and r["err"] == 0.0
    import scipy.linalg as sl
    ref = sl.expm(-0.1 * A.toarray()) @ x
    assert np.linalg.norm(r["y"] - ref) / np.linalg.norm(ref) < 1e-12


def test_zero_vector(orc):
    T = orc.Csr.from_scipy(-matrices.laplacian_1d(20))
    r = orc.krylov("LANCZOS", orc.serial("EXP", "GENPADE", 1.0), T, np.zeros(20), 1e-6)
    assert r["info"] == 0 and r["iter"] == 0 and not np.any(r["y"])


def lanczos_breakdown_case():
    """Path graph on nodes 0-1-2 with unit diagonal (plus isolated nodes), x = e_1:
    every Krylov quantity is an exact small integer and the fourth basis vector is 0."""
    import scipy.sparse as sp
    n = 20
    A = sp.lil_matrix((n, n))
    A[0, 1] = A[1, 0] = A[1, 2] = A[2, 1] = 1.0
    A[0, 0] = A[1, 1] = A[2, 2] = 1.0
    for i in range(3, n):
        A[i, i] = float(i)
    x = np.zeros(n)
    x[0] = 1.0
    return A.tocsr(), x


def test_lanczos_breakdown(orc):
    """|beta| < 1e-16 at the top of iteration 4 ends the loop with itx = 3 and f is
    taken on T(1:itx-1) (psfun_d_lanczos.f90:225-230, :330-362)."""
    A, x = lanczos_breakdown_case()
    r = orc.krylov("LANCZOS", orc.serial("EXP", "GENPADE", 1.0), orc.Csr.from_scipy(A), x, 1e-14, itmax=10,
                   istop=2)
    assert r["info"] == 0 and r["iter"] == 3


def test_arnoldi_breakdown_istop1(orc):
    """Arnoldi has no breakdown test: h(4,3) == 0 makes the estimate 0 and the step converges."""
    A, x = lanczos_breakdown_case()
    r = orc.krylov("ARNOLDI", orc.serial("EXP", "GENPADE", 1.0), orc.Csr.from_scipy(A), x, 1e-14, itmax=10)
    assert r["info"] == 0 and r["iter"] == 3
    import scipy.linalg as sl
    assert np.linalg.norm(r["y"][:3] - sl.expm(A.toarray()[:3, :3])[:, 0][:3]) > 0  # reference drops one term


def test_null_projected_matrix_is_error(orc):
    """H(1,1) == 0 with GENPADE: DGPADM stops on a null matrix (dgpadm.f:84); 4011 here."""
    import scipy.sparse as sp
    A = sp.lil_matrix((5, 5))
    A[0, 1] = A[1, 0] = 1.0
    x = np.zeros(5)
    x[0] = 1.0
    r = orc.krylov("ARNOLDI", orc.serial("EXP", "GENPADE", 1.0), orc.Csr.from_scipy(A.tocsr()), x, 1e-14, itmax=6)
    assert r["info"] == 4011


def test_lanczos_eigenvector_is_error(orc):
    """x an eigenvector: breakdown at iteration 2 leaves T(1:0); the reference stops in
    DGPADM ('null H'), the restatement returns 4011."""
    import scipy.sparse as sp
    A = sp.diags(np.arange(1.0, 11.0)).tocsr()
    x = np.zeros(10)
    x[3] = 1.0
    r = orc.krylov("LANCZOS", orc.serial("EXP", "GENPADE", 1.0), orc.Csr.from_scipy(A), x, 1e-14, itmax=10,
                   istop=2)
    assert r["info"] == 4011


@pytest.mark.parametrize("fname,variant,k", [("PHI", "", 1), ("EXP", "SASQ", 1), ("EXP", "CHBHES", 1)])
def test_arnoldi_other_functions(orc, fname, variant, k):
    A = matrices.convdiff_2d(24)
    x = matrices.unit(np.random.default_rng(1).standard_normal(A.shape[0]))
    t = -1e-3
    r = orc.krylov("ARNOLDI", orc.serial(fname, variant, t, phiorder=k), orc.Csr.from_scipy(A), x, 1e-12,
                   itmax=60, drop_last=False)
    assert r["info"] == 0
    ref = orc.dense_phi1_times(A.toarray(), x, t) if fname == "PHI" else orc.dense_expm_times(A.toarray(), x, t)
    assert np.linalg.norm(r["y"] - ref) / np.linalg.norm(ref) < 1e-9


def test_oracle_saiarnoldi_tau0_matches_dense_expm(orc):
    """psfun_d_saiarnoldi restated (krylov/rational/psfun_d_sai.f90): with
    tau = 0 the shift quirk is void and a converged estimate gives exp(A)x on a
    negative definite A (the inner CG solves A w = v)."""
    import scipy.linalg as sl
    A = -matrices.laplacian_2d(20)
    x = matrices.unit(np.random.default_rng(3).standard_normal(A.shape[0]))
    ref = sl.expm(A.toarray()) @ x
    for prec in ("NONE", "DIAG"):
        r = orc.saiarnoldi(orc.serial("EXP", "GENPADE", 1.0), orc.Csr.from_scipy(A), x, 1e-10, tau=0.0,
                           prec=prec, istop=1, itmax=40)
        assert r["info"] == 0 and r["err"] < 1e-10
        assert np.linalg.norm(r["y"] - ref) <= 1e-8 * np.linalg.norm(ref)


def test_oracle_saiarnoldi_reference_quirks(orc):
    """Only hcomp(1,1) is shifted (`do j=1,i-1,i`, :296-298), so tau != 0 does
    not converge to exp(A)x; without a converged estimate the assembly applies f
    to H itself (:346-368).  The restatement keeps both."""
    import scipy.linalg as sl
    A = -matrices.laplacian_2d(20)
    x = matrices.unit(np.random.default_rng(3).standard_normal(A.shape[0]))
    ref = sl.expm(A.toarray()) @ x
    r = orc.saiarnoldi(orc.serial("EXP", "GENPADE", 1.0), orc.Csr.from_scipy(A), x, 1e-10, tau=-1.0, istop=1,
                       itmax=40)
    assert r["info"] == 0 and np.linalg.norm(r["y"] - ref) > 0.1 * np.linalg.norm(ref)
    r2 = orc.saiarnoldi(orc.serial("EXP", "GENPADE", 1.0), orc.Csr.from_scipy(A), x, 1e-10, tau=0.0, istop=2,
                        itmax=40)
    assert r2["info"] == 0 and r2["iter"] == 39


def test_oracle_spmv_on_power_law_rows(orc):
    # the checker of the GPU row-splitting tests: exact on integer data,
    # against scipy, whatever the row lengths
    A = matrices.skewed_rows(30000, alpha=1.2, seed=31, integer=True)
    x = np.random.default_rng(32).integers(-5, 6, size=A.shape[0]).astype(np.float64)
    y0 = np.random.default_rng(33).integers(-5, 6, size=A.shape[0]).astype(np.float64)
    oa = orc.Csr.from_scipy(A)
    assert np.array_equal(orc.spmv(oa, x), A @ x)
    assert np.array_equal(orc.spmv(oa, x, alpha=2.0, beta=-3.0, y=y0), 2.0 * (A @ x) - 3.0 * y0)
