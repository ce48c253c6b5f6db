"""Batched f(t A) X (one persistent launch for many uneven instances) against
the plain per-instance drop-in calls and the oracle, pair by pair."""
import numpy as np
import pytest

from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu


def make_items(seed=0, R=4):
    rng = np.random.default_rng(seed)
    mats = [matrices.laplacian_2d(s) for s in (9, 23, 40, 31)]
    mats += [matrices.rgg_knn_laplacian(n, 8, rng) for n in (300, 1500, 4100)]
    out = []
    for A in mats:
        X = rng.standard_normal((R, A.shape[0]))
        t = float(rng.uniform(0.01, 1.0))
        out.append((A, X, t))
    return out


def plain(A, x, t, eps, itmax, istop=1):
    import psfun_gb300 as pg
    fun = pg.PsfunDSerial()
    fun.set("FNAME", "EXP")
    fun.set("VARIANT", "CHBSYM")
    meth = pg.PsfunDKrylov()
    meth.set("KNAME", "LANCZOS")
    return meth.apply(fun, pg.CsrMatrix.from_scipy(t * A), x, eps, itmax=itmax, istop=istop)


def oracle_spread(orc, A, x, t, eps, itmax, istop):
    """Relative change of the oracle's result when only its reduction order
    changes (1 against 4 OpenMP threads): the FP64 reproducibility floor of the
    case.  It is ~1e-15 for the converged cases and reaches ~3e-10 on the kNN
    graph with n = 4100, whose 39 unconverged steps amplify rounding."""
    prev = orc.set_threads(0)
    ys = []
    for th in (1, 4):
        orc.set_threads(th)
        ys.append(orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), orc.Csr.from_scipy(t * A), x, eps,
                             itmax=itmax, istop=istop)["y"])
    orc.set_threads(prev)
    return np.linalg.norm(ys[0] - ys[1]) / np.linalg.norm(ys[0])


@pytest.mark.parametrize("istop", [1, 2])
@pytest.mark.parametrize("R", [1, 4])
def test_batch_matches_plain(lib, orc, istop, R):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    eps, itmax = 1e-8, 40
    items = make_items(1, R)
    handles = []
    for A, X, t in items:
        a = pg.CsrMatrix.from_scipy(A)
        Xd = torch.tensor(X, device="cuda")
        Yd = torch.zeros_like(Xd)
        handles.append((a, Xd, Yd, t))
    fun = pg.PsfunDSerial()
    fun.set("FNAME", "EXP")
    fun.set("VARIANT", "CHBSYM")
    meth = pg.PsfunDKrylov()
    meth.set("KNAME", "LANCZOS")
    info, infos, iters, errs = pg.krylov_batch(meth, fun, handles, eps, itmax=itmax, istop=istop)
    torch.cuda.synchronize()
    assert info == 0 and not infos.any()
    for k, ((A, X, t), (a, Xd, Yd, _)) in enumerate(zip(items, handles)):
        Y = Yd.cpu().numpy()
        for q in range(R):
            r = plain(A, X[q], t, eps, itmax, istop)
            o = orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), orc.Csr.from_scipy(t * A), X[q], eps,
                           itmax=itmax, istop=istop)
            assert r.info == 0 and o["info"] == 0
            assert iters[k, q] == r.iter == o["iter"], (k, q, iters[k, q], r.iter, o["iter"])
            # 1e-10, or 10x the oracle's own reduction-order spread where that is larger
            tol = max(1e-10, 10 * oracle_spread(orc, A, X[q], t, eps, itmax, istop))
            assert np.linalg.norm(Y[q] - r.y) <= tol * np.linalg.norm(r.y), (k, q, tol)
            assert np.linalg.norm(Y[q] - o["y"]) <= tol * np.linalg.norm(o["y"]), (k, q, tol)


def skewed_laplacian(n, seed):
    """Graph Laplacian (+ 0.1 I) of a power-law degree graph, scaled to
    spectral radius <= 1: rows of 2..~8000 entries."""
    import scipy.sparse as sp
    B = abs(matrices.skewed_rows(n, alpha=1.3, seed=seed))
    S = (B + B.T).tocsr()
    d = np.asarray(S.sum(axis=1)).ravel()
    L = (sp.diags(d + 0.1) - S).tocsr()
    L.sort_indices()
    return (-(0.5 / d.max()) * L).tocsr()


@pytest.mark.parametrize("mapping", [-1, 0, 1, 2])
def test_batch_mappings_skewed_rows(lib, orc, mapping):
    # every SpMM mapping of the batch (and the autotuner's pick) on instances
    # with power-law row lengths beside regular ones, against the plain calls
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    eps, itmax, R = 1e-8, 30, 2
    rng = np.random.default_rng(40)
    mats = [skewed_laplacian(n, 41 + k) for k, n in enumerate((3000, 20000, 70000))]
    mats.append(-0.2 * matrices.laplacian_2d(50))
    items, handles = [], []
    for A in mats:
        X = rng.standard_normal((R, A.shape[0]))
        items.append((A, X))
        handles.append((pg.CsrMatrix.from_scipy(A), torch.tensor(X, device="cuda"),
                        torch.zeros((R, A.shape[0]), dtype=torch.float64, device="cuda"), 1.0))
    fun = pg.PsfunDSerial()
    fun.set("FNAME", "EXP")
    fun.set("VARIANT", "CHBSYM")
    meth = pg.PsfunDKrylov()
    meth.set("KNAME", "LANCZOS")
    assert meth.set("BATCHMAP", mapping) == 0
    info, infos, iters, errs = pg.krylov_batch(meth, fun, handles, eps, itmax=itmax, istop=1)
    torch.cuda.synchronize()
    assert info == 0 and not infos.any()
    for k, ((A, X), (_, _, Yd, _)) in enumerate(zip(items, handles)):
        Y = Yd.cpu().numpy()
        for q in range(R):
            r = plain(A, X[q], 1.0, eps, itmax, 1)
            assert r.info == 0 and iters[k, q] == r.iter, (k, q)
            assert np.linalg.norm(Y[q] - r.y) <= 1e-10 * np.linalg.norm(r.y), (k, q)
    assert meth.set("BATCHMAP", 3) == 111 and meth.set("BATCHMAP", -2) == 111


def test_batch_zero_rhs_and_errors(lib):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    A = matrices.laplacian_2d(12)
    a = pg.CsrMatrix.from_scipy(A)
    X = torch.zeros((2, 144), dtype=torch.float64, device="cuda")
    X[1] = 1.0
    Y = torch.full_like(X, 7.0)
    fun = pg.PsfunDSerial()
    fun.set("VARIANT", "CHBSYM")
    meth = pg.PsfunDKrylov()
    meth.set("KNAME", "LANCZOS")
    info, infos, iters, errs = pg.krylov_batch(meth, fun, [(a, X, Y, 0.5)], 1e-10, itmax=30)
    torch.cuda.synchronize()
    assert info == 0 and iters[0, 0] == 0 and not Y[0].any()
    assert torch.isfinite(Y[1]).all()
    fun.set("VARIANT", "GENPADE")
    assert pg.krylov_batch(meth, fun, [(a, X, Y, 0.5)], 1e-10, itmax=30)[0] == 111
    fun.set("VARIANT", "CHBSYM")
    meth.set("KNAME", "SAIARNOLDI")
    assert pg.krylov_batch(meth, fun, [(a, X, Y, 0.5)], 1e-10, itmax=30)[0] == 111


def test_quadrature_batch_matches_single(lib):
    """Quadrature items (each its own HHT poles and weights, f(z) = z^{-1/2}) in
    one batched launch against the single-instance quadrature sum, pair by
    pair: the same number of Lanczos steps and the same result (1e-10)."""
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    rng = np.random.default_rng(5)
    mats = [(matrices.laplacian_2d(s), s) for s in (12, 30, 47)]
    mats += [(matrices.rgg_knn_laplacian(n, 8, rng, shift=0.5), None) for n in (500, 3000)]
    items = []
    for k, (A, side) in enumerate(mats):
        if side is not None:
            lam = lambda j: 4.0 * np.sin(np.pi * j / (2.0 * (side + 1))) ** 2
            bounds = [2 * lam(1), 2 * lam(side)]
        else:
            bounds = [0.5, float(abs(A).sum(axis=1).max())]
        q = pg.PsfunZQuadrature()
        assert q.computepoles(pg.hhtmethod1, lambda z: 1.0 / np.sqrt(z), 12 + 4 * k, rparams=bounds) == 0
        a = pg.CsrMatrix.from_scipy(A)
        q.setmatrix(a)
        X = torch.tensor(rng.standard_normal((2, A.shape[0])), device="cuda")
        items.append((a, X, torch.zeros_like(X), q))
    info, infos, iters, errs = pg.quadrature_batch(items, eps=1e-10, itmax=2000)
    torch.cuda.synchronize()
    assert info == 0 and not infos.any()
    for k, (a, X, Y, q) in enumerate(items):
        for r in range(2):
            y1, inf1, it1, err1 = q.apply(X[r].cpu().numpy(), eps=1e-10, itmax=2000)
            assert inf1 == 0
            assert iters[k, r] == it1, (k, r, iters[k, r], it1)
            yb = Y[r].cpu().numpy()
            assert np.linalg.norm(yb - y1) <= 1e-10 * np.linalg.norm(y1), (k, r)
            assert errs[k, r] < 1e-10


def test_quadrature_batch_refuses_nonsymmetric(lib):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    q = pg.PsfunZQuadrature()
    assert q.computepoles(pg.hhtmethod1, lambda z: 1.0 / np.sqrt(z), 8, rparams=[1.0, 10.0]) == 0
    a = pg.CsrMatrix.from_scipy(matrices.convdiff_2d(8))
    X = torch.ones((1, 64), dtype=torch.float64, device="cuda")
    assert pg.quadrature_batch([(a, X, torch.zeros_like(X), q)])[0] == 111


def arnoldi_items(R, seed=11):
    rng = np.random.default_rng(seed)
    mats = [matrices.convdiff_2d(N) for N in (12, 20, 33)]
    mats += [matrices.laplacian_2d(15), matrices.rgg_knn_laplacian(500, 8, rng)]
    out = []
    for A in mats:
        X = rng.standard_normal((R, A.shape[0]))
        t = -float(rng.uniform(1.0, 8.0)) / float(abs(A).sum(axis=1).max())
        out.append((A, X, t))
    return out


@pytest.mark.parametrize("istop", [1, 2])
@pytest.mark.parametrize("fname,variant", [("EXP", "GENPADE"), ("PHI", "")])
def test_batch_arnoldi_matches_plain(lib, orc, istop, fname, variant):
    """KNAME 'ARNOLDI' in the batched launch (nonsymmetric and symmetric
    instances, two right-hand sides each) against the plain Arnoldi drop-in
    on t A for every pair and against the oracle: the same iteration count
    and the same result (1e-10)."""
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    eps, itmax, R = 1e-10, 40, 2
    items = arnoldi_items(R)
    handles = []
    for A, X, t in items:
        Xd = torch.tensor(X, device="cuda")
        handles.append((pg.CsrMatrix.from_scipy(A), Xd, torch.zeros_like(Xd), t))
    fun = pg.PsfunDSerial()
    assert fun.set("FNAME", fname) == 0 and fun.set("VARIANT", variant) == 0
    meth = pg.PsfunDKrylov()
    meth.set("KNAME", "ARNOLDI")
    info, infos, iters, errs = pg.krylov_batch(meth, fun, handles, eps, itmax=itmax, istop=istop)
    torch.cuda.synchronize()
    assert info == 0 and not infos.any(), (info, infos, lib.psfun_gpu_last_error())
    for k, ((A, X, t), (a, Xd, Yd, _)) in enumerate(zip(items, handles)):
        Y = Yd.cpu().numpy()
        fk = pg.PsfunDSerial()
        fk.set("FNAME", fname); fk.set("VARIANT", variant); fk.set("SCALING", t)
        for q in range(R):
            r = pg.PsfunDKrylov()
            r.set("KNAME", "ARNOLDI")
            p = r.apply(fk, a, X[q], eps, itmax=itmax, istop=istop)
            o = orc.krylov("ARNOLDI", orc.serial(fname, variant, t), orc.Csr.from_scipy(A), X[q], eps, itmax=itmax,
                           istop=istop)
            assert p.info == 0 and o["info"] == 0
            assert iters[k, q] == p.iter == o["iter"], (k, q, iters[k, q], p.iter, o["iter"])
            assert np.linalg.norm(Y[q] - p.y) <= 1e-10 * np.linalg.norm(p.y), (k, q)
            assert np.linalg.norm(Y[q] - o["y"]) <= 1e-10 * np.linalg.norm(o["y"]), (k, q)


def test_batch_arnoldi_zero_rhs_and_userf(lib):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    a = pg.CsrMatrix.from_scipy(matrices.convdiff_2d(10))
    X = torch.zeros((2, 100), dtype=torch.float64, device="cuda")
    X[1] = 1.0
    Y = torch.full_like(X, 7.0)
    fun = pg.PsfunDSerial()
    fun.set("VARIANT", "GENPADE")
    meth = pg.PsfunDKrylov()
    meth.set("KNAME", "ARNOLDI")
    info, infos, iters, errs = pg.krylov_batch(meth, fun, [(a, X, Y, -1e-3)], 1e-10, itmax=30)
    torch.cuda.synchronize()
    assert info == 0 and iters[0, 0] == 0 and not Y[0].any() and torch.isfinite(Y[1]).all()
    fu = pg.PsfunDSerial()
    fu.set("FNAME", "USERF"); fu.set("VARIANT", "SYM"); fu.set("FPOINTER", lambda v, k: float(np.exp(v)))
    assert pg.krylov_batch(meth, fu, [(a, X, Y, -1e-3)], 1e-10, itmax=30)[0] == 111
