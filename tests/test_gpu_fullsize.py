"""Full-size parity of the benchmark configurations, through the C-ABI:

  laplace3d_lanczos  exp(-0.05 A) x on the 128^3 7-point Laplacian, Lanczos
                     m = 80: against the exact Kronecker-sum evaluation (<= 1e-8)
                     and against the oracle's Lanczos (<= 1e-10).
  convdiff_phi1      phi_1(-1e-3 A) x on the 2048^2 convection-diffusion
                     operator, Arnoldi m = 60 (istop 2): against the oracle's
                     Arnoldi (<= 1e-10); the truncation error of m = 60 and the
                     convergence of larger m against the exact evaluation
                     (Sylvester solve with the 1-D factors); on the 512^2
                     instance, m = 260 against the exact value (<= 1e-9).
  uneven_batch       all 64 instances x 4 right-hand sides of the batched
                     launch against the oracle, pair by pair (identical
                     iteration counts; 1e-10 or 10x the oracle's own
                     reduction-order spread).

Reference semantics: krylov/polynomial/psfun_d_lanczos.f90:219-377 and
krylov/polynomial/psfun_d_arnoldi.f90:199-329.
"""
import numpy as np
import pytest

from oracle import exact
from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def serial(fname, variant, scaling, phiorder=1):
    import psfun_gb300 as pg
    fun = pg.PsfunDSerial()
    assert fun.set("FNAME", fname) == 0 and fun.set("VARIANT", variant) == 0
    assert fun.set("SCALING", float(scaling)) == 0 and fun.set("PHIORDER", phiorder) == 0
    return fun


def method(kname):
    import psfun_gb300 as pg
    meth = pg.PsfunDKrylov()
    assert meth.set("KNAME", kname) == 0
    return meth


def test_laplace3d_128_lanczos(lib, orc):
    import psfun_gb300 as pg
    p = matrices.laplace3d_lanczos()
    t, m = p.params["t"], p.params["m"]
    # the reference's Lanczos ignores fun%scaling (psfun_d_lanczos.f90:172-173):
    # exp(-tA)x is computed on the matrix -tA
    At = (-t * p.A).tocsr()
    r = method("LANCZOS").apply(serial("EXP", "CHBSYM", 1.0), pg.CsrMatrix.from_scipy(At), p.x, 1e-12, itmax=m,
                                istop=2)
    assert r.info == 0
    y_exact = exact.laplacian_3d_apply(128, p.x, lambda L: np.exp(-t * L))
    assert rel(r.y, y_exact) <= 1e-8, rel(r.y, y_exact)
    o = orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), orc.Csr.from_scipy(At), p.x, 1e-12, itmax=m,
                   istop=2)
    assert o["info"] == 0 and o["iter"] == r.iter
    assert rel(r.y, o["y"]) <= 1e-10, rel(r.y, o["y"])


@pytest.fixture(scope="module")
def convdiff():
    p = matrices.convdiff_phi1()
    return p, exact.convdiff_phi1(2048, p.x, p.params["t"])


def test_convdiff_2048_arnoldi_phi1_vs_oracle(lib, orc, convdiff):
    import psfun_gb300 as pg
    p, y_exact = convdiff
    t, m = p.params["t"], p.params["m"]
    fun = serial("PHI", "", -t, 1)
    r = method("ARNOLDI").apply(fun, pg.CsrMatrix.from_scipy(p.A), p.x, 1e-12, itmax=m, istop=2)
    assert r.info == 0
    o = orc.krylov("ARNOLDI", orc.serial("PHI", "", -t, phiorder=1), orc.Csr.from_scipy(p.A), p.x, 1e-12, itmax=m,
                   istop=2)
    assert o["info"] == 0 and o["iter"] == r.iter
    assert rel(r.y, o["y"]) <= 1e-10, rel(r.y, o["y"])
    # the m = 60 result is a truncated Krylov approximation: the GPU and the
    # oracle carry the same truncation error against the exact phi_1
    e_gpu, e_orc = rel(r.y, y_exact), rel(o["y"], y_exact)
    assert abs(e_gpu - e_orc) <= 1e-9 * max(e_orc, 1e-300) + 1e-12, (e_gpu, e_orc)
    print(f"convdiff 2048^2 phi_1 m=60: rel. error vs exact {e_gpu:.3e} (oracle {e_orc:.3e})")


def test_convdiff_2048_arnoldi_phi1_converges_to_exact(lib, convdiff):
    """Larger Krylov dimensions approach the exact phi_1(-1e-3 A) x on the
    2048^2 operator (||tA|| ~ 3.4e4 and A is far from normal, so a polynomial
    Krylov space needs several hundred steps: 60 -> 0.80, 500 -> 1.3e-3)."""
    import torch
    import psfun_gb300 as pg
    p, y_exact = convdiff
    t = p.params["t"]
    a = pg.CsrMatrix.from_scipy(p.A)
    xd = torch.tensor(p.x, device="cuda")
    errs = {}
    for m in (120, 300, 500):
        r = method("ARNOLDI").apply(serial("PHI", "", -t, 1), a, xd, 1e-12, itmax=m, istop=2)
        assert r.info == 0
        errs[m] = rel(r.y.cpu().numpy(), y_exact)
    print("convdiff 2048^2 phi_1 rel. error vs exact by m:", {k: f"{v:.2e}" for k, v in errs.items()})
    assert errs[500] < errs[300] < errs[120]
    assert errs[500] <= 5e-3, errs


def test_convdiff_512_arnoldi_phi1_equals_exact(lib, orc):
    """On the 512^2 instance of the same operator (||tA|| ~ 2.1e3) Arnoldi with
    m = 260 reaches the exact phi_1(-1e-3 A) x, and matches the oracle."""
    import psfun_gb300 as pg
    N, t, m = 512, 1e-3, 260
    A = matrices.convdiff_2d(N)
    x = matrices.unit(np.random.default_rng(1).standard_normal(N * N))
    r = method("ARNOLDI").apply(serial("PHI", "", -t, 1), pg.CsrMatrix.from_scipy(A), x, 1e-12, itmax=m, istop=2)
    assert r.info == 0
    e = rel(r.y, exact.convdiff_phi1(N, x, t))
    assert e <= 1e-9, e
    o = orc.krylov("ARNOLDI", orc.serial("PHI", "", -t, phiorder=1), orc.Csr.from_scipy(A), x, 1e-12, itmax=m,
                   istop=2)
    assert o["iter"] == r.iter and rel(r.y, o["y"]) <= 1e-10, rel(r.y, o["y"])


def test_uneven_batch_full_vs_oracle(lib, orc):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    probs = matrices.uneven_batch()
    eps, itmax = 1e-8, 60
    items = []
    for pr in probs:
        X = torch.tensor(pr.x, device="cuda")
        items.append((pg.CsrMatrix.from_scipy(pr.A), X, torch.zeros_like(X), -pr.params["t"]))
    info, infos, iters, errs = pg.krylov_batch(method("LANCZOS"), serial("EXP", "CHBSYM", 1.0), items, eps,
                                               itmax=itmax, istop=1)
    torch.cuda.synchronize()
    assert info == 0 and not infos.any()
    fo = orc.serial("EXP", "CHBSYM", 1.0)
    worst = 0.0
    for k, (pr, (a, X, Y, t)) in enumerate(zip(probs, items)):
        ot = orc.Csr.from_scipy((t * pr.A).tocsr())
        Yh = Y.cpu().numpy()
        for q in range(pr.x.shape[0]):
            o = orc.krylov("LANCZOS", fo, ot, pr.x[q], eps, itmax=itmax, istop=1)
            assert o["info"] == 0
            assert iters[k, q] == o["iter"], (k, q, pr.name, iters[k, q], o["iter"])
            d = rel(Yh[q], o["y"])
            if d > 1e-10:
                # the oracle's own FP64 reduction-order spread (1 against 4 threads)
                prev = orc.set_threads(1)
                y1 = orc.krylov("LANCZOS", fo, ot, pr.x[q], eps, itmax=itmax, istop=1)["y"]
                orc.set_threads(4)
                y4 = orc.krylov("LANCZOS", fo, ot, pr.x[q], eps, itmax=itmax, istop=1)["y"]
                orc.set_threads(prev)
                assert d <= 10 * rel(y1, y4), (k, q, pr.name, d, rel(y1, y4))
            worst = max(worst, d)
    print(f"uneven batch 64 x 4: worst rel. diff vs oracle {worst:.2e}")
