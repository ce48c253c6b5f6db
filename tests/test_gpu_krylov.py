"""Arnoldi / Lanczos f(A)x on the GPU against the oracle (relative 2-norm
difference <= 1e-10, identical iteration counts), the committed fixtures, and
the reference's error behaviour."""
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu
FIX = np.load(Path(__file__).parent / "golden" / "driver_scenarios.npz")
TOL = 1e-10


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def run_gpu(kname, fname, variant, scaling, A, x, eps, itmax=200, istop=1, phiorder=1, keeplast=False, f=None):
    import psfun_gb300 as pg
    fun = pg.PsfunDSerial()
    assert fun.set("FNAME", fname) == 0 and fun.set("VARIANT", variant) == 0
    assert fun.set("SCALING", float(scaling)) == 0 and fun.set("PHIORDER", phiorder) == 0
    if f is not None:
        assert fun.set("FPOINTER", f) == 0
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", kname) == 0
    if keeplast:
        assert meth.set("KEEPLAST", 1) == 0
    return meth.apply(fun, pg.CsrMatrix.from_scipy(A), x, eps, itmax=itmax, istop=istop)


def run_orc(orc, kname, fname, variant, scaling, A, x, eps, itmax=200, istop=1, phiorder=1, keeplast=False, f=None):
    return orc.krylov(kname, orc.serial(fname, variant, scaling, phiorder=phiorder, f=f), orc.Csr.from_scipy(A), x,
                      eps, itmax=itmax, istop=istop, drop_last=not keeplast)


def test_laplace2d_100_arnoldi(lib):
    p = matrices.laplace2d_expm()
    r = run_gpu("ARNOLDI", "EXP", "GENPADE", -1.0, p.A, p.x, 1e-10, itmax=50)
    assert r.info == 0
    assert r.iter == int(FIX["lap2d_arn_iter"]) == 18
    assert rel(r.y, FIX["lap2d_arn_y"]) <= TOL
    assert rel(r.y, FIX["lap2d_dense_y"]) <= 1e-10
    assert abs(r.err - float(FIX["lap2d_arn_err"])) <= 1e-6 * float(FIX["lap2d_arn_err"])
    assert np.allclose(r.res, FIX["lap2d_arn_res"], rtol=1e-6, atol=0)


def test_laplace2d_100_lanczos(lib):
    p = matrices.laplace2d_expm()
    r = run_gpu("LANCZOS", "EXP", "CHBSYM", 1.0, -p.A, p.x, 1e-10, itmax=50)
    assert r.info == 0 and r.iter == int(FIX["lap2d_lz_iter"])
    assert rel(r.y, FIX["lap2d_lz_y"]) <= TOL
    assert rel(r.y, FIX["lap2d_dense_y"]) <= 1e-10


@pytest.mark.parametrize("kname,variant,fix", [("ARNOLDI", "GENPADE", "arn"), ("LANCZOS", "CHBSYM", "lz")])
def test_driver_scenarios(lib, kname, variant, fix):
    """arnolditest / lanczostest on laplacian.mtx with the driver's eps 1e-6, itmax 100, istop 1, x = 1."""
    T = -matrices.laplacian_1d(50)
    r = run_gpu(kname, "EXP", variant, 1.0, T, np.ones(50), 1e-6, itmax=100)
    assert r.info == 0 and r.iter == int(FIX[f"{fix}_iter"])
    assert rel(r.y, FIX[f"{fix}_y"]) <= TOL


ARN_VARIANTS = [("EXP", "GENPADE", 1), ("EXP", "CHBHES", 1), ("EXP", "CHBGEN", 1), ("EXP", "CHBSYM", 1),
                ("EXP", "SASQ", 1), ("EXP", "TAYLOR", 1), ("PHI", "", 1), ("PHI", "", 2)]


@pytest.mark.parametrize("fname,variant,k", ARN_VARIANTS)
@pytest.mark.parametrize("istop", [1, 2])
def test_arnoldi_variants_vs_oracle(lib, orc, fname, variant, k, istop):
    A = matrices.convdiff_2d(20)
    x = matrices.unit(np.random.default_rng(5).standard_normal(A.shape[0]))
    t = -2e-4
    itmax = 40 if istop == 2 else 60
    g = run_gpu("ARNOLDI", fname, variant, t, A, x, 1e-10, itmax=itmax, istop=istop, phiorder=k)
    o = run_orc(orc, "ARNOLDI", fname, variant, t, A, x, 1e-10, itmax=itmax, istop=istop, phiorder=k)
    assert g.info == 0 and o["info"] == 0
    assert g.iter == o["iter"]
    assert rel(g.y, o["y"]) <= TOL


@pytest.mark.parametrize("variant", ["GENPADE", "CHBSYM", "CHBGEN", "CHBHES", "SASQ"])
@pytest.mark.parametrize("istop", [1, 2])
def test_lanczos_variants_vs_oracle(lib, orc, variant, istop):
    A = -0.3 * matrices.laplacian_2d(24)
    x = matrices.unit(np.random.default_rng(6).standard_normal(A.shape[0]))
    g = run_gpu("LANCZOS", "EXP", variant, 1.0, A, x, 1e-11, itmax=45, istop=istop)
    o = run_orc(orc, "LANCZOS", "EXP", variant, 1.0, A, x, 1e-11, itmax=45, istop=istop)
    assert g.info == 0 and o["info"] == 0 and g.iter == o["iter"]
    assert rel(g.y, o["y"]) <= TOL


def test_lanczos_skewed_graph_vs_oracle(lib, orc):
    # a graph Laplacian with power-law degrees: the persistent Lanczos' SpMV
    # sums the high-degree rows across a warp, into its fused epilogue
    B = abs(matrices.skewed_rows(30000, alpha=1.3, seed=26))
    S = (B + B.T).tocsr()
    d = np.asarray(S.sum(axis=1)).ravel()
    L = (sp.diags(d + 0.1) - S).tocsr()
    L.sort_indices()
    A = (-(0.5 / d.max()) * L).tocsr()
    x = matrices.unit(np.random.default_rng(27).standard_normal(A.shape[0]))
    for istop in (1, 2):
        g = run_gpu("LANCZOS", "EXP", "CHBSYM", 1.0, A, x, 1e-11, itmax=40, istop=istop)
        o = run_orc(orc, "LANCZOS", "EXP", "CHBSYM", 1.0, A, x, 1e-11, itmax=40, istop=istop)
        assert g.info == 0 and o["info"] == 0 and g.iter == o["iter"]
        assert rel(g.y, o["y"]) <= TOL


def test_lanczos_ignores_scaling(lib, orc):
    """Lanczos drops fun%scaling (psfun_d_lanczos.f90:172-173,198): f(A)x is returned."""
    A = -matrices.laplacian_2d(16)
    x = matrices.unit(np.ones(256))
    g1 = run_gpu("LANCZOS", "EXP", "GENPADE", 1.0, A, x, 1e-12, itmax=40)
    g2 = run_gpu("LANCZOS", "EXP", "GENPADE", 0.25, A, x, 1e-12, itmax=40)
    assert g1.info == g2.info == 0 and rel(g1.y, g2.y) <= 1e-14


def test_keeplast(lib, orc):
    p = matrices.laplace2d_expm()
    g = run_gpu("ARNOLDI", "EXP", "GENPADE", -1.0, p.A, p.x, 1e-10, itmax=50, keeplast=True)
    o = run_orc(orc, "ARNOLDI", "EXP", "GENPADE", -1.0, p.A, p.x, 1e-10, itmax=50, keeplast=True)
    assert g.info == 0 and g.iter == o["iter"] and rel(g.y, o["y"]) <= TOL
    assert rel(g.y, FIX["lap2d_dense_y"]) < rel(FIX["lap2d_arn_y"], FIX["lap2d_dense_y"])


@pytest.mark.parametrize("kname", ["ARNOLDI", "LANCZOS"])
def test_userf_sym(lib, orc, kname):
    A = -0.5 * matrices.laplacian_2d(12)
    x = matrices.unit(np.random.default_rng(8).standard_normal(144))
    f = lambda v, k: float(np.exp(v))
    g = run_gpu(kname, "USERF", "SYM", 1.0, A, x, 1e-10, itmax=40, f=f)
    o = run_orc(orc, kname, "USERF", "SYM", 1.0, A, x, 1e-10, itmax=40, f=f)
    assert g.info == 0 and o["info"] == 0 and g.iter == o["iter"]
    assert rel(g.y, o["y"]) <= TOL


def test_errors(lib):
    import psfun_gb300 as pg
    T = -matrices.laplacian_1d(30)
    x = np.ones(30)
    assert run_gpu("ARNOLDI", "EXP", "GENPADE", 1.0, T, x, 1e-6, istop=3).info == 5001
    assert run_gpu("LANCZOS", "EXP", "GENPADE", 1.0, T, x, 1e-6, istop=0).info == 5001
    assert run_gpu("ARNOLDI", "EXP", "GENPADE", 1.0, T, x, 1e-6, itmax=1).info == 4011
    assert run_gpu("ARNOLDI", "EXP", "EXPOKIT", 1.0, T, x, 1e-6).info == 4011
    assert run_gpu("ARNOLDI", "exp", "GENPADE", 1.0, T, x, 1e-6).info == 4011
    assert run_gpu("NOSUCH", "EXP", "GENPADE", 1.0, T, x, 1e-6).info == 111
    # kname is upper-cased before the dispatch (psfun_d_krylov_mod.F90:254)
    assert run_gpu("lanczos", "EXP", "GENPADE", 1.0, T, x, 1e-6).info == 0


def test_zero_vector(lib):
    T = -matrices.laplacian_1d(30)
    r = run_gpu("ARNOLDI", "EXP", "GENPADE", 1.0, T, np.zeros(30), 1e-6)
    assert r.info == 0 and r.iter == 0 and not np.any(r.y)


def test_lanczos_breakdown_cases(lib, orc):
    from test_oracle_krylov import lanczos_breakdown_case
    A, x = lanczos_breakdown_case()
    g = run_gpu("LANCZOS", "EXP", "GENPADE", 1.0, A, x, 1e-14, itmax=10, istop=2)
    o = run_orc(orc, "LANCZOS", "EXP", "GENPADE", 1.0, A, x, 1e-14, itmax=10, istop=2)
    assert g.info == 0 and g.iter == o["iter"] == 3 and rel(g.y, o["y"]) <= TOL
    D = sp.diags(np.arange(1.0, 11.0)).tocsr()
    e = np.zeros(10)
    e[3] = 1.0
    assert run_gpu("LANCZOS", "EXP", "GENPADE", 1.0, D, e, 1e-14, itmax=10, istop=2).info == 4011


def test_arnoldi_exact_breakdown_istop1(lib, orc):
    """Arnoldi has no breakdown test; with istop 1 the estimate is 0 and the step converges."""
    from test_oracle_krylov import lanczos_breakdown_case
    A, x = lanczos_breakdown_case()
    g = run_gpu("ARNOLDI", "EXP", "GENPADE", 1.0, A, x, 1e-14, itmax=10, istop=1)
    o = run_orc(orc, "ARNOLDI", "EXP", "GENPADE", 1.0, A, x, 1e-14, itmax=10, istop=1)
    assert g.info == 0 and o["info"] == 0 and g.iter == o["iter"] == 3 and rel(g.y, o["y"]) <= TOL
    # istop 2: the native path stops at the exact breakdown and uses the whole invariant subspace
    g2 = run_gpu("ARNOLDI", "EXP", "GENPADE", 1.0, A, x, 1e-14, itmax=10, istop=2)
    import scipy.linalg as sl
    ref = sl.expm(A.toarray()) @ x
    assert g2.info == 0 and g2.iter == 3 and rel(g2.y, ref) < 1e-13


def test_null_projected_matrix_is_error(lib):
    import scipy.sparse as sp
    A = sp.lil_matrix((5, 5))
    A[0, 1] = A[1, 0] = 1.0
    x = np.zeros(5)
    x[0] = 1.0
    assert run_gpu("ARNOLDI", "EXP", "GENPADE", 1.0, A.tocsr(), x, 1e-14, itmax=6).info == 4011


def test_device_api_matches_host_api(lib):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    p = matrices.laplace2d_expm()
    fun = pg.PsfunDSerial()
    fun.set("FNAME", "EXP"); fun.set("VARIANT", "GENPADE"); fun.set("SCALING", -1.0)
    meth = pg.PsfunDKrylov()
    a = pg.CsrMatrix.from_scipy(p.A)
    rh = meth.apply(fun, a, p.x, 1e-10, itmax=50)
    rd = meth.apply(fun, a, torch.tensor(p.x, device="cuda"), 1e-10, itmax=50)
    torch.cuda.synchronize()
    assert rh.info == rd.info == 0 and rh.iter == rd.iter
    assert np.array_equal(rd.y.cpu().numpy(), rh.y)  # same kernels, same order: bitwise


def test_repeatable_bitwise(lib):
    p = matrices.laplace2d_expm()
    r1 = run_gpu("ARNOLDI", "EXP", "GENPADE", -1.0, p.A, p.x, 1e-10, itmax=50)
    r2 = run_gpu("ARNOLDI", "EXP", "GENPADE", -1.0, p.A, p.x, 1e-10, itmax=50)
    assert np.array_equal(r1.y, r2.y)


def test_semigroup_property_3d(lib):
    """exp(-tA) exp(-tA) x == exp(-2tA) x on a 64^3 Laplacian (size-independent check)."""
    A = matrices.laplacian_3d(64)
    x = matrices.unit(np.random.default_rng(1).standard_normal(A.shape[0]))
    import psfun_gb300 as pg
    a = pg.CsrMatrix.from_scipy(-A)
    meth = pg.PsfunDKrylov()
    meth.set("KNAME", "LANCZOS")
    f1 = pg.PsfunDSerial(); f1.set("VARIANT", "CHBSYM")
    r1 = meth.apply(f1, pg.CsrMatrix.from_scipy(-0.05 * A), x, 1e-12, itmax=80)
    r2 = meth.apply(f1, pg.CsrMatrix.from_scipy(-0.05 * A), r1.y, 1e-12, itmax=80)
    r3 = meth.apply(f1, pg.CsrMatrix.from_scipy(-0.1 * A), x, 1e-12, itmax=80)
    assert r1.info == r2.info == r3.info == 0
    assert rel(r2.y, r3.y) < 1e-10
    assert np.linalg.norm(r1.y) < 1.0


@pytest.mark.parametrize("side", [300, 2100])
def test_arnoldi_both_mgs_paths(lib, orc, side):
    """Arnoldi keeps a block's rows of w in shared memory while they fit
    (n <= ~4.3M rows on 152 SMs) and in global memory beyond: 2-D Laplacians
    with n = 90,000 and n = 4,410,000 exercise both MGS kernels against the
    oracle (fixed Krylov dimension 12)."""
    A = matrices.laplacian_2d(side)
    x = matrices.unit(np.random.default_rng(side).standard_normal(A.shape[0]))
    g = run_gpu("ARNOLDI", "EXP", "GENPADE", -0.01, A, x, 1e-12, itmax=12, istop=2)
    orc.set_threads(0)
    o = run_orc(orc, "ARNOLDI", "EXP", "GENPADE", -0.01, A, x, 1e-12, itmax=12, istop=2)
    assert g.info == 0 and o["info"] == 0 and g.iter == o["iter"]
    assert rel(g.y, o["y"]) <= TOL


def test_itrace_log(lib, capfd):
    """itrace > 0: the convergence log (header, every itrace-th estimate, end
    line) under the reference's method name KNAME+FNAME+VARIANT."""
    import psfun_gb300 as pg
    A = -matrices.laplacian_2d(30)
    x = matrices.unit(np.random.default_rng(4).standard_normal(A.shape[0]))
    fun = pg.PsfunDSerial()
    assert fun.set("VARIANT", "GENPADE") == 0
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", "arnoldi") == 0
    capfd.readouterr()
    r = meth.apply(fun, pg.CsrMatrix.from_scipy(A), x, 1e-10, itmax=80, itrace=3, istop=1)
    out = capfd.readouterr().out.splitlines()
    assert r.info == 0
    lines = [l for l in out if l.startswith("ARNOLDI+EXP+GENPADE:")]
    assert "error estimate" in lines[0]
    its = [int(l.split()[1]) for l in lines[1:-1]]
    assert its == list(range(3, r.iter, 3))
    for l in lines[1:-1]:
        it = int(l.split()[1])
        assert float(l.split()[2]) == pytest.approx(r.res[it], rel=1e-7)
    assert f"converged after {r.iter} iterations" in lines[-1]
    # itrace 0: silent
    meth.apply(fun, pg.CsrMatrix.from_scipy(A), x, 1e-10, itmax=80, istop=1)
    assert "ARNOLDI+" not in capfd.readouterr().out


@pytest.mark.parametrize("kname,variant,istop", [("LANCZOS", "CHBSYM", 2), ("ARNOLDI", "GENPADE", 1)])
def test_pinned_host_vectors_in_place(lib, kname, variant, istop):
    """Pinned, mapped host vectors are read and written by the kernels in place
    (no staging copies): the same result, bit for bit, as pageable arrays;
    x sharing memory with y is staged first."""
    import torch
    import psfun_gb300 as pg
    A = -matrices.laplacian_2d(60)
    n = A.shape[0]
    x = matrices.unit(np.random.default_rng(9).standard_normal(n))
    a = pg.CsrMatrix.from_scipy(A)
    fun = pg.PsfunDSerial()
    assert fun.set("VARIANT", variant) == 0
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", kname) == 0
    ref = meth.apply(fun, a, x.copy(), 1e-10, itmax=60, istop=istop)
    xp = torch.tensor(x).pin_memory()
    yp = torch.zeros(n, dtype=torch.float64).pin_memory()
    r = meth.apply(fun, a, xp.numpy(), 1e-10, itmax=60, istop=istop, y=yp.numpy())
    assert r.info == 0 and r.iter == ref.iter
    assert np.array_equal(yp.numpy(), ref.y)
    # in place: y is x
    r2 = meth.apply(fun, a, xp.numpy(), 1e-10, itmax=60, istop=istop, y=xp.numpy())
    assert r2.info == 0 and np.array_equal(xp.numpy(), ref.y)


@pytest.mark.parametrize("variant", ["CHBSYM", "GENPADE"])
def test_lanczos_istop1_estimate_monitors(lib, orc, variant):
    """istop = 1 Lanczos in one launch, its a posteriori estimates on four
    monitor blocks that take the iterations in turn: every combination of a
    short Krylov dimension (the monitors with no iteration, or one) and an
    eps that converges at each early iteration matches the oracle's serial
    loop (same iteration count and estimate, y within 1e-10), and the breakdown
    case stops the estimates where psfun_d_lanczos.f90:225-230 does."""
    A = -0.5 * matrices.laplacian_2d(20)
    x = matrices.unit(np.random.default_rng(21).standard_normal(A.shape[0]))
    for itmax in (2, 3, 4, 5, 6, 9, 14):
        for eps in (1e-1, 1e-3, 1e-6, 1e-9, 1e-13):
            g = run_gpu("LANCZOS", "EXP", variant, 1.0, A, x, eps, itmax=itmax, istop=1)
            o = run_orc(orc, "LANCZOS", "EXP", variant, 1.0, A, x, eps, itmax=itmax, istop=1)
            # (itmax 2 without convergence leaves a null projected matrix:
            # 4011 from both)
            assert g.info == o["info"], (itmax, eps, g.info, o["info"])
            if o["info"] != 0:
                continue
            assert g.iter == o["iter"], (itmax, eps, g.iter, o["iter"])
            # the estimate divides by yk's last entry, which rounding moves
            # relative to its own small size
            assert abs(g.err - o["err"]) <= 1e-3 * abs(o["err"]) + 1e-15, (itmax, eps, g.err, o["err"])
            assert rel(g.y, o["y"]) <= TOL, (itmax, eps)
    from test_oracle_krylov import lanczos_breakdown_case
    B, xb = lanczos_breakdown_case()
    g = run_gpu("LANCZOS", "EXP", variant, 1.0, B, xb, 1e-14, itmax=10, istop=1)
    o = run_orc(orc, "LANCZOS", "EXP", variant, 1.0, B, xb, 1e-14, itmax=10, istop=1)
    assert g.info == o["info"] == 0 and g.iter == o["iter"] and rel(g.y, o["y"]) <= TOL


def test_arnoldi_istop1_concurrent_estimates_stop(lib, orc):
    """istop = 1 Arnoldi: the estimates run beside the steps and the first
    converged one stops the steps still queued (at their first grid barrier,
    all blocks alike).  Krylov dimensions 2..12 and eps from 1e-1 to 1e-12 on
    a nonsymmetric operator match the oracle's serial loop (same iteration
    count, y within 1e-10), and a solve after an early stop is unaffected."""
    A = -1e-3 * matrices.convdiff_2d(24)
    x = matrices.unit(np.random.default_rng(22).standard_normal(A.shape[0]))
    for itmax in (2, 3, 5, 8, 12):
        for eps in (1e-1, 1e-4, 1e-8, 1e-12):
            g = run_gpu("ARNOLDI", "EXP", "GENPADE", 1.0, A, x, eps, itmax=itmax, istop=1)
            o = run_orc(orc, "ARNOLDI", "EXP", "GENPADE", 1.0, A, x, eps, itmax=itmax, istop=1)
            assert g.info == o["info"], (itmax, eps, g.info, o["info"])
            if o["info"] != 0:
                continue
            assert g.iter == o["iter"], (itmax, eps, g.iter, o["iter"])
            assert rel(g.y, o["y"]) <= TOL, (itmax, eps)
    g = run_gpu("ARNOLDI", "EXP", "GENPADE", 1.0, A, x, 1e-12, itmax=40, istop=2)
    o = run_orc(orc, "ARNOLDI", "EXP", "GENPADE", 1.0, A, x, 1e-12, itmax=40, istop=2)
    assert g.info == 0 and g.iter == o["iter"] and rel(g.y, o["y"]) <= TOL
