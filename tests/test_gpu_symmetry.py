"""The symmetry check of a CSR handle, and the entry points that rely on a
symmetric matrix (the batched Lanczos launch and the quadrature sum) refusing
a nonsymmetric one with 111."""
import numpy as np
import pytest
import scipy.sparse as sp

from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu


def test_is_symmetric(lib):
    import psfun_gb300 as pg
    assert pg.CsrMatrix.from_scipy(matrices.laplacian_2d(9)).is_symmetric()
    assert pg.CsrMatrix.from_scipy(matrices.rgg_knn_laplacian(300, 8, np.random.default_rng(0))).is_symmetric()
    assert not pg.CsrMatrix.from_scipy(matrices.convdiff_2d(9)).is_symmetric()
    # same pattern, one value differs by one ulp
    A = matrices.laplacian_2d(7).tocsr()
    A.data[5] = np.nextafter(A.data[5], 0.0)
    assert not pg.CsrMatrix.from_scipy(A).is_symmetric()
    # a symmetric matrix stored with unsorted rows
    B = matrices.laplacian_1d(6).tocsr()
    irp, ja, val = B.indptr.copy(), B.indices.copy(), B.data.copy()
    for i in range(6):
        s, e = irp[i], irp[i + 1]
        ja[s:e], val[s:e] = ja[s:e][::-1].copy(), val[s:e][::-1].copy()
    assert pg.CsrMatrix(irp, ja, val).is_symmetric()
    # pattern-symmetric only: an explicit zero on one side
    C = sp.csr_matrix(np.array([[2.0, 0.0], [1.0, 2.0]]))
    C2 = sp.csr_matrix((np.array([2.0, 0.0, 1.0, 2.0]), np.array([0, 1, 0, 1]), np.array([0, 2, 4])), shape=(2, 2))
    assert not pg.CsrMatrix.from_scipy(C).is_symmetric()
    assert not pg.CsrMatrix(C2.indptr, C2.indices, C2.data).is_symmetric()


def test_batch_and_quadrature_refuse_nonsymmetric(lib):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    A = matrices.convdiff_2d(10)
    a = pg.CsrMatrix.from_scipy(A)
    X = torch.ones((1, 100), dtype=torch.float64, device="cuda")
    Y = torch.zeros_like(X)
    fun = pg.PsfunDSerial()
    fun.set("VARIANT", "CHBSYM")
    meth = pg.PsfunDKrylov()
    meth.set("KNAME", "LANCZOS")
    assert pg.krylov_batch(meth, fun, [(a, X, Y, -0.01)], 1e-8, itmax=30)[0] == 111
    assert b"symmetric" in lib.psfun_gpu_last_error()
    q = pg.PsfunZQuadrature()
    assert q.computepoles(pg.hhtmethod1, lambda z: 1.0 / np.sqrt(z), 8, rparams=[1.0, 10.0]) == 0
    q.setmatrix(a)
    _, info, _, _ = q.apply(np.ones(100))
    assert info == 111
    # the same calls on a symmetric matrix run
    L = pg.CsrMatrix.from_scipy(matrices.laplacian_2d(10))
    assert pg.krylov_batch(meth, fun, [(L, X, Y, -0.01)], 1e-8, itmax=30)[0] == 0
    q.setmatrix(L)
    assert q.apply(np.ones(100))[1] == 0
