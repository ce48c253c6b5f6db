"""Failure behaviour on the GPU without faulting it: bounded device waits that
expire (a wait that nothing completes), an allocation the device cannot
satisfy, NaN inputs and an undersized residual buffer.  After each, the
library must still give correct results."""
import ctypes as C
import time

import numpy as np
import pytest

from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu


def lanczos_ok(orc, n1=20):
    """A normal solve after a failure: Lanczos exp(-A)x on a 2-D Laplacian
    against the oracle (relative 1e-10)."""
    import psfun_gb300 as pg
    A = -matrices.laplacian_2d(n1)
    x = matrices.unit(np.random.default_rng(11).standard_normal(A.shape[0]))
    fun = pg.PsfunDSerial()
    assert fun.set("VARIANT", "CHBSYM") == 0
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", "LANCZOS") == 0
    r = meth.apply(fun, pg.CsrMatrix.from_scipy(A), x, 1e-10, itmax=60, istop=1)
    o = orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), orc.Csr.from_scipy(A), x, 1e-10, itmax=60, istop=1)
    assert r.info == 0 and r.iter == o["iter"]
    assert np.linalg.norm(r.y - o["y"]) <= 1e-10 * np.linalg.norm(o["y"])


@pytest.mark.parametrize("which", [0, 1])
def test_bounded_wait_expires_and_reports(lib, orc, which):
    """A grid barrier short of one arrival (0) and an mbarrier phase nobody
    completes (1) give up after the 2 s limit with status 9002."""
    t0 = time.perf_counter()
    rc = lib.psfun_gpu_selftest_wait(which)
    dt = time.perf_counter() - t0
    assert rc == 9002, lib.psfun_gpu_last_error()
    assert b"expired" in lib.psfun_gpu_last_error()
    assert 1.5 <= dt <= 30.0
    lanczos_ok(orc)


def test_device_allocation_failure(lib, orc):
    """A basis larger than HBM (itmax 5e7 on n = 1000: ~410 GB) fails with
    psb_err_alloc_dealloc_ (4000) and the next call succeeds."""
    import psfun_gb300 as pg
    A = -matrices.laplacian_1d(1000)
    a = pg.CsrMatrix.from_scipy(A)
    fun = pg.PsfunDSerial()
    assert fun.set("VARIANT", "CHBSYM") == 0
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", "LANCZOS") == 0
    x = np.ones(1000)
    y = np.zeros(1000)
    it, err, nres = C.c_int(0), C.c_double(0.0), C.c_int(0)
    dp = lambda v: v.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    info = lib.psfun_gpu_d_krylov_apply(meth.handle, fun.handle, a.handle, dp(y), dp(x), 1e-10, 50_000_000, 0, 2,
                                        C.byref(it), C.byref(err), None, 0, C.byref(nres))
    assert info == 4000
    assert b"cudaMalloc" in lib.psfun_gpu_last_error()
    # the same handle recovers with a normal Krylov dimension
    r = meth.apply(fun, a, x, 1e-10, itmax=60, istop=1)
    assert r.info == 0 and np.all(np.isfinite(r.y))
    lanczos_ok(orc)


@pytest.mark.parametrize("kname", ["ARNOLDI", "LANCZOS"])
def test_nan_input_returns(lib, orc, kname):
    """A NaN in x propagates like the reference's arithmetic (no check there):
    the call returns (no hang) with NaN in y or a failure status."""
    import psfun_gb300 as pg
    A = -matrices.laplacian_2d(20)
    x = np.ones(A.shape[0])
    x[7] = np.nan
    fun = pg.PsfunDSerial()
    assert fun.set("VARIANT", "GENPADE") == 0
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", kname) == 0
    for istop in (1, 2):
        r = meth.apply(fun, pg.CsrMatrix.from_scipy(A), x, 1e-10, itmax=30, istop=istop)
        assert r.info != 0 or np.isnan(r.y).any()
    lanczos_ok(orc)


def test_nan_input_cg(lib, orc):
    import psfun_gb300 as pg
    A = matrices.laplacian_2d(20)
    b = np.ones(A.shape[0])
    b[3] = np.nan
    x, info, it, err = pg.psb_krylov("CG", pg.CsrMatrix.from_scipy(A), "DIAG", b, 1.0, 0.5, np.zeros_like(b), 1e-10,
                                     itmax=200, istop=2)
    assert info != 0 or np.isnan(x).any() or not np.isfinite(err)
    lanczos_ok(orc)


def test_undersized_residual_buffer(lib):
    """res_cap below iter + 1: the first res_cap entries of the history."""
    import psfun_gb300 as pg
    A = -matrices.laplacian_2d(30)
    x = matrices.unit(np.random.default_rng(2).standard_normal(A.shape[0]))
    a = pg.CsrMatrix.from_scipy(A)
    fun = pg.PsfunDSerial()
    assert fun.set("VARIANT", "GENPADE") == 0
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", "ARNOLDI") == 0
    full = meth.apply(fun, a, x, 1e-10, itmax=80, istop=1)
    assert full.info == 0 and full.iter > 5
    y = np.zeros_like(x)
    res = np.full(4, -1.0)
    it, err, nres = C.c_int(0), C.c_double(0.0), C.c_int(0)
    dp = lambda v: v.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    info = lib.psfun_gpu_d_krylov_apply(meth.handle, fun.handle, a.handle, dp(y), dp(x), 1e-10, 80, 0, 1,
                                        C.byref(it), C.byref(err), dp(res), 4, C.byref(nres))
    assert info == 0 and it.value == full.iter and nres.value == 4
    assert np.array_equal(res, full.res[:4])
    assert np.array_equal(y, full.y)
