"""Adjoint of y = exp(tA(theta)) x on grid-graph Laplacians.

Oracles: the dense FP64 Frechet derivative (expm of the block matrix
[[M, E], [0, M]], and the equivalent eigen divided differences) on a 32 x 32
grid, and central finite differences (h = 1e-6) on 64 random coordinates at the
full 512 x 512 size.  The torch.autograd.Function below exists in the tests
only; the library itself has no torch dependency in its C-ABI."""
import numpy as np
import pytest
import scipy.linalg as sl

from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu


def edge_pattern(A, ei, ej):
    """CSR positions of (a,a), (b,b), (a,b), (b,a) for every edge."""
    A = A.tocsr()
    A.sort_indices()
    def pos(r, c):
        lo, hi = A.indptr[r], A.indptr[r + 1]
        k = lo + np.searchsorted(A.indices[lo:hi], c)
        assert A.indices[k] == c
        return k
    P = np.zeros((len(ei), 4), dtype=np.int64)
    for e, (a, b) in enumerate(zip(ei, ej)):
        P[e] = (pos(a, a), pos(b, b), pos(a, b), pos(b, a))
    return P


def theta_grad(gvals, P):
    """dL/dtheta_e from dL/dA on the pattern: dA/dtheta_e = E_aa + E_bb - E_ab - E_ba."""
    return gvals[P[:, 0]] + gvals[P[:, 1]] - gvals[P[:, 2]] - gvals[P[:, 3]]


def small_case(N=32, seed=4):
    rng = np.random.default_rng(seed)
    ei, ej = matrices.grid_edges(N)
    th = rng.lognormal(0.0, 0.7, len(ei))
    A = matrices.graph_laplacian(N * N, ei, ej, th)
    x = rng.standard_normal(N * N)
    g = rng.standard_normal(N * N)
    return A, ei, ej, th, x, g


def test_adjoint_small_vs_dense_frechet(lib):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    A, ei, ej, th, x, g = small_case()
    t = -0.1
    a = pg.CsrMatrix.from_scipy(A)
    r = pg.expm_adjoint(a, t, torch.tensor(x, device="cuda"), torch.tensor(g, device="cuda"))
    torch.cuda.synchronize()
    Ad = A.toarray()
    E = sl.expm(t * Ad)
    y = r["y"].cpu().numpy()
    assert np.linalg.norm(y - E @ x) / np.linalg.norm(E @ x) < 1e-12
    assert np.linalg.norm(r["grad_x"].cpu().numpy() - E.T @ g) / np.linalg.norm(E.T @ g) < 1e-12
    gt_ref = g @ (Ad @ (E @ x))
    assert abs(r["grad_t"] - gt_ref) <= 1e-11 * abs(gt_ref)
    # exact Frechet derivative through the eigendecomposition (divided differences)
    lam, Q = np.linalg.eigh(Ad)
    el = np.exp(t * lam)
    D = np.subtract.outer(t * lam, t * lam)
    with np.errstate(divide="ignore", invalid="ignore"):
        Phi = np.where(np.abs(D) > 1e-12, np.subtract.outer(el, el) / D, el[:, None] * np.ones_like(D))
    gh, xh = Q.T @ g, Q.T @ x
    W = Q[ei] - Q[ej]                                      # (edges, n) rows w_e = Q^T (e_a - e_b)
    ref = t * np.einsum("ei,ij,ej->e", W * gh, Phi, W * xh, optimize=True)
    P = edge_pattern(A, ei, ej)
    got = theta_grad(r["grad_vals"].cpu().numpy(), P)
    assert np.max(np.abs(got - ref)) <= 1e-10 * np.max(np.abs(ref))
    # the block-matrix oracle on a few edges: g^T L(tA, t E_e) x
    for e in (0, 17, len(ei) // 2, len(ei) - 1):
        Ee = np.zeros_like(Ad)
        a_, b_ = ei[e], ej[e]
        Ee[a_, a_] = Ee[b_, b_] = 1.0
        Ee[a_, b_] = Ee[b_, a_] = -1.0
        n = Ad.shape[0]
        B = np.zeros((2 * n, 2 * n))
        B[:n, :n] = t * Ad
        B[n:, n:] = t * Ad
        B[:n, n:] = t * Ee
        Lf = sl.expm(B)[:n, n:]
        assert abs(got[e] - g @ Lf @ x) <= 1e-10 * np.max(np.abs(ref))


def test_adjoint_recompute_equals_stored(lib):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    A, ei, ej, th, x, g = small_case(24, 7)
    a = pg.CsrMatrix.from_scipy(A)
    xd, gd = torch.tensor(x, device="cuda"), torch.tensor(g, device="cuda")
    r1 = pg.expm_adjoint(a, -0.1, xd, gd, recompute=False)
    r2 = pg.expm_adjoint(a, -0.1, xd, gd, recompute=True)
    torch.cuda.synchronize()
    assert torch.equal(r1["grad_vals"], r2["grad_vals"])
    assert torch.equal(r1["grad_x"], r2["grad_x"])


def dense_frechet_grad(Ad, t, x, g):
    """dL/dA for L = g^T exp(tA) x: t [expm([[tA^T, g x^T], [0, tA^T]])]_12."""
    n = Ad.shape[0]
    B = np.zeros((2 * n, 2 * n))
    B[:n, :n] = t * Ad.T
    B[n:, n:] = t * Ad.T
    B[:n, n:] = np.outer(g, x)
    return t * sl.expm(B)[:n, n:]


@pytest.mark.parametrize("N,t", [(24, -1e-3), (32, -2e-3)])
def test_adjoint_nonsymmetric_vs_dense_frechet(lib, N, t):
    """Nonsymmetric A (2-D upwind convection-diffusion): y and grad_x =
    exp(tA^T) g from Arnoldi on A and A^T, grad_t, and dL/dA on the pattern
    through the Van Loan block exponential, against the dense block-expm
    Frechet derivative."""
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    A = matrices.convdiff_2d(N)
    rng = np.random.default_rng(N)
    x, g = rng.standard_normal(N * N), rng.standard_normal(N * N)
    a = pg.CsrMatrix.from_scipy(A)
    assert not a.is_symmetric()
    xd, gd = torch.tensor(x, device="cuda"), torch.tensor(g, device="cuda")
    r = pg.expm_adjoint(a, t, xd, gd, eps=1e-15, itmax=200)
    torch.cuda.synchronize()
    Ad = A.toarray()
    E = sl.expm(t * Ad)
    y = r["y"].cpu().numpy()
    assert np.linalg.norm(y - E @ x) / np.linalg.norm(E @ x) < 1e-12
    gx = r["grad_x"].cpu().numpy()
    assert np.linalg.norm(gx - E.T @ g) / np.linalg.norm(E.T @ g) < 1e-12
    gt_ref = g @ (Ad @ (E @ x))
    assert abs(r["grad_t"] - gt_ref) <= 1e-11 * abs(gt_ref)
    G = dense_frechet_grad(Ad, t, x, g)
    Ac = A.tocsr()
    rows = np.repeat(np.arange(N * N), np.diff(Ac.indptr))
    ref = G[rows, Ac.indices]
    got = r["grad_vals"].cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-10 * np.max(np.abs(ref))
    # recomputing the forward basis gives the same gradients
    r2 = pg.expm_adjoint(a, t, xd, gd, eps=1e-15, itmax=200, recompute=True)
    torch.cuda.synchronize()
    assert torch.equal(r["grad_vals"], r2["grad_vals"]) and torch.equal(r["grad_x"], r2["grad_x"])


class ExpmAction:
    """Test-harness torch.autograd.Function: y = exp(t A(theta)) x."""

    @staticmethod
    def make(ei, ej, n):
        import torch
        import psfun_gb300 as pg

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, theta, x, t):
                A = matrices.graph_laplacian(n, ei, ej, theta.detach().cpu().numpy())
                a = pg.CsrMatrix.from_scipy(A)
                r = pg.expm_adjoint(a, float(t), x.detach(), None, want=("y",))
                ctx.save_for_backward(theta, x, t)
                ctx.a, ctx.P = a, edge_pattern(A, ei, ej)
                return r["y"]

            @staticmethod
            def backward(ctx, gy):
                theta, x, t = ctx.saved_tensors
                r = pg.expm_adjoint(ctx.a, float(t), x.detach(), gy.contiguous())
                gv = r["grad_vals"]
                P = torch.as_tensor(ctx.P, device=gv.device)
                gth = gv[P[:, 0]] + gv[P[:, 1]] - gv[P[:, 2]] - gv[P[:, 3]]
                return gth, r["grad_x"], torch.tensor(r["grad_t"], dtype=torch.float64, device=x.device)

        return Fn


def test_autograd_full_size_vs_finite_differences(lib):
    """512 x 512 grid, L = 1/2 ||exp(-0.1 A(theta)) x - y*||^2.

    Every check uses central differences at steps d and 2d combined by
    Richardson extrapolation (the d^2 term cancels), so the step can be large
    enough (d = 1e-3) that the FD's own FP64 rounding floor, about
    eps * L / d (L ~ 4.5e3 here, i.e. ~1e-9), sits far below the gradients:
    64 random coordinates of theta and 16 of x are held to
    |fd - grad| <= 1e-6 |grad| + 20 eps L / d, and directional derivatives
    along random dense directions to 1e-6 relative."""
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    cfg = matrices.grid_graph_adjoint()
    N, ei, ej = cfg["N"], cfg["ei"], cfg["ej"]
    n = N * N
    Fn = ExpmAction.make(ei, ej, n)
    dev = "cuda"
    x = torch.tensor(cfg["x"], device=dev)
    t0 = -cfg["t"]
    t = torch.tensor(t0, dtype=torch.float64, device=dev, requires_grad=True)
    ystar = pg.expm_adjoint(pg.CsrMatrix.from_scipy(matrices.graph_laplacian(n, ei, ej, cfg["theta_star"])),
                            t0, x, None, want=("y",))["y"]
    theta = torch.tensor(cfg["theta"], device=dev, requires_grad=True)
    xv = x.clone().requires_grad_(True)
    y = Fn.apply(theta, xv, t)
    loss = 0.5 * torch.sum((y - ystar) ** 2)
    loss.backward()
    Lval = float(loss.detach())
    h = 1e-6
    floor = 20 * 2.220446049250313e-16 * Lval / h

    def y_of(th, xx, tt):
        # fixed Krylov dimension: y(theta) is then a smooth function
        A = matrices.graph_laplacian(n, ei, ej, th)
        return pg.expm_adjoint(pg.CsrMatrix.from_scipy(A), tt, xx, None, want=("y",), eps=0.0, itmax=48)["y"]

    def fd_of(yp, ym):  # L(+) - L(-) = 1/2 (y+ - y-) . (y+ + y- - 2 y*), over 2h
        return float(0.5 * torch.dot(yp - ym, yp + ym - 2 * ystar)) / (2 * h)

    th0 = cfg["theta"].copy()
    gth = theta.grad.cpu().numpy()
    rng = np.random.default_rng(11)

    # Richardson extrapolation of central differences at d and 2d
    def dirfd(yfun, d):
        f1 = fd_of(*yfun(d)) * (h / d)
        f2 = fd_of(*yfun(2 * d)) * (h / (2 * d))
        return (4 * f1 - f2) / 3

    d = 1e-3
    floor = 20 * 2.220446049250313e-16 * Lval / d
    rel = []
    for e in rng.choice(len(ei), size=64, replace=False):
        unit = np.zeros(len(ei))
        unit[e] = 1.0
        fd = dirfd(lambda dd: (y_of(th0 + dd * unit, x, t0), y_of(th0 - dd * unit, x, t0)), d)
        assert abs(fd - gth[e]) <= 1e-6 * abs(gth[e]) + floor, (e, fd, gth[e])
        rel.append(abs(fd - gth[e]) / abs(gth[e]))

    for k in range(3):
        v = rng.standard_normal(len(ei))
        fd = dirfd(lambda d: (y_of(th0 + d * v, x, t0), y_of(th0 - d * v, x, t0)), 1e-3)
        ad = float(np.dot(gth, v))
        assert abs(fd - ad) <= 1e-6 * abs(ad), (k, fd, ad)
    gx = xv.grad.cpu().numpy()
    for j in rng.choice(n, size=16, replace=False):
        ej_ = torch.zeros_like(x)
        ej_[j] = 1.0
        fd = dirfd(lambda dd: (y_of(th0, x + dd * ej_, t0), y_of(th0, x - dd * ej_, t0)), d)
        assert abs(fd - gx[j]) <= 1e-6 * abs(gx[j]) + floor, (j, fd, gx[j])
    v = torch.tensor(rng.standard_normal(n), device=dev)
    fd = dirfd(lambda d: (y_of(th0, x + d * v, t0), y_of(th0, x - d * v, t0)), 1e-3)
    ad = float(torch.dot(xv.grad, v))
    assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)
    fd = dirfd(lambda d: (y_of(th0, x, t0 + d), y_of(th0, x, t0 - d)), 1e-4)
    assert abs(fd - float(t.grad)) <= 1e-6 * abs(float(t.grad)), (fd, float(t.grad))
    print(f"FD per-coordinate relative error: median {np.median(rel):.2e}, max {np.max(rel):.2e}; "
          f"FP64 floor {floor:.1e}")
