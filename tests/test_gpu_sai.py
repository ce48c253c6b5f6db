"""Shift-and-invert Arnoldi (KNAME 'SAIARNOLDI', psfun_d_saiarnoldi,
krylov/rational/psfun_d_sai.f90) on the GPU against the oracle: the inner
solves are the GPU CG, the outer loop, Gram-Schmidt, estimate and assembly the
GPU kernels.  Both sides solve the inner systems only to the outer eps, so the
two results agree to a few times eps, not to rounding: 1e-8 relative."""
import numpy as np
import pytest

from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu
TOL = 1e-8


def run_gpu(A, x, eps, tau, istop, itmax, prec="NONE", fname="EXP", variant="GENPADE"):
    import psfun_gb300 as pg
    fun = pg.PsfunDSerial()
    assert fun.set("FNAME", fname) == 0 and fun.set("VARIANT", variant) == 0
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", "SAIARNOLDI") == 0
    assert meth.set("TAU", float(tau)) == 0 and meth.set("PREC", prec) == 0
    return meth.apply(fun, pg.CsrMatrix.from_scipy(A), x, eps, itmax=itmax, istop=istop)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("tau,istop,prec", [(0.0, 1, "NONE"), (0.0, 1, "DIAG"), (-1.0, 1, "NONE"),
                                            (0.0, 2, "NONE"), (0.0, 1, "BJAC")])
def test_sai_vs_oracle(lib, orc, tau, istop, prec):
    A = -matrices.laplacian_2d(20)
    x = matrices.unit(np.random.default_rng(3).standard_normal(A.shape[0]))
    g = run_gpu(A, x, 1e-10, tau, istop, 40, prec)
    o = orc.saiarnoldi(orc.serial("EXP", "GENPADE", 1.0), orc.Csr.from_scipy(A), x, 1e-10, tau=tau, prec=prec,
                       istop=istop, itmax=40)
    assert g.info == 0 and o["info"] == 0 and g.iter == o["iter"]
    assert rel(g.y, o["y"]) <= TOL


def test_sai_converges_to_expm(lib):
    import scipy.linalg as sl
    A = -matrices.laplacian_2d(24)
    x = matrices.unit(np.random.default_rng(5).standard_normal(A.shape[0]))
    g = run_gpu(A, x, 1e-10, 0.0, 1, 60, "DIAG")
    ref = sl.expm(A.toarray()) @ x
    assert g.info == 0 and g.err < 1e-10 and rel(g.y, ref) <= 1e-8


def test_sai_errors(lib):
    import psfun_gb300 as pg
    A = -matrices.laplacian_2d(8)
    x = np.ones(64)
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", "SAIARNOLDI") == 0
    assert meth.set("PREC", "AMG") == 111
    fun = pg.PsfunDSerial()
    fun.set("FNAME", "USERF"); fun.set("VARIANT", "SYM"); fun.set("FPOINTER", lambda v, k: float(np.exp(v)))
    assert meth.apply(fun, pg.CsrMatrix.from_scipy(A), x, 1e-8, itmax=10).info == 111
    fun2 = pg.PsfunDSerial(); fun2.set("VARIANT", "GENPADE")
    assert meth.apply(fun2, pg.CsrMatrix.from_scipy(A), x, 1e-8, itmax=10, istop=3).info == 5001


def test_precinit_precbuild_diag(lib):
    """precinit('DIAG') + precbuild(a) (psfun_d_prec_init / psfun_d_prec_build)
    builds the Jacobi preconditioner before apply; the result is identical to
    building it lazily on the first inner solve."""
    import psfun_gb300 as pg
    A = -matrices.laplacian_2d(20)
    x = matrices.unit(np.random.default_rng(5).standard_normal(A.shape[0]))
    lazy = run_gpu(A, x, 1e-10, 0.0, 1, 40, "DIAG")
    fun = pg.PsfunDSerial()
    assert fun.set("VARIANT", "GENPADE") == 0
    meth = pg.PsfunDKrylov()
    a = pg.CsrMatrix.from_scipy(A)
    assert meth.set("KNAME", "SAIARNOLDI") == 0
    assert meth.precinit("DIAG") == 0 and meth.precbuild(a) == 0
    r = meth.apply(fun, a, x, 1e-10, itmax=40, istop=1)
    assert r.info == 0 and lazy.info == 0 and r.iter == lazy.iter
    assert np.array_equal(r.y, lazy.y)


def test_precinit_precbuild_bjac(lib):
    """precinit('BJAC') + precbuild(a): the block-Jacobi ILU(0) factors built
    before apply give the same result as building them on the first inner
    solve."""
    import psfun_gb300 as pg
    A = -matrices.laplacian_2d(20)
    x = matrices.unit(np.random.default_rng(5).standard_normal(A.shape[0]))
    lazy = run_gpu(A, x, 1e-10, 0.0, 1, 40, "BJAC")
    fun = pg.PsfunDSerial()
    assert fun.set("VARIANT", "GENPADE") == 0
    meth = pg.PsfunDKrylov()
    a = pg.CsrMatrix.from_scipy(A)
    assert meth.set("KNAME", "SAIARNOLDI") == 0
    assert meth.precinit("BJAC") == 0 and meth.precbuild(a) == 0
    r = meth.apply(fun, a, x, 1e-10, itmax=40, istop=1)
    assert r.info == 0 and lazy.info == 0 and r.iter == lazy.iter
    assert np.array_equal(r.y, lazy.y)
