"""Seeded synthetic workloads and MatrixMarket ingest.

The reference's drivers read MatrixMarket files (examples/polynomial/arnolditest.F90:111-125)
and ship one fixture, a 50 x 50 1-D Laplacian (examples/polynomial/laplacian.mtx).
The benchmark problems are synthetic and seeded (numpy default_rng):

  laplace2d_expm      2-D 5-point Dirichlet Laplacian 100 x 100, stencil [-1,-1,4,-1,-1],
                      x ~ U[-1,1]^n (seed 0) normalised; y = exp(-A) x
  laplace3d_lanczos   3-D 7-point Laplacian 128^3 (unscaled), x ~ N(0,1) (seed 1) normalised;
                      y = exp(-0.05 A) x by Lanczos, m = 80
  convdiff_phi1       2-D convection-diffusion 2048^2, -Lap u + beta.grad u, beta = (50, 25),
                      first-order upwind, h = 1/2049, scaled by h^-2 / h^-1; y = phi_1(-1e-3 A) x
  laplace3d_invsqrt   3-D 7-point Laplacian 96^3, x ~ N(0,1) (seed 2); y = A^{-1/2} x by the
                      HHT rule with N = 24 and the analytic spectrum bounds
  uneven_batch        64 uneven instances (seed 3), 4 right-hand sides each
  grid_graph_adjoint  512^2 grid-graph Laplacian with lognormal(0,0.7) conductivities (seed 4)
  skewed_rows         power-law row lengths (alpha 1.5, 4..4000 entries; seed 5) for the SpMV's
                      row splitting
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp


def _tridiag(n: int, lo: float, d: float, up: float) -> sp.csr_matrix:
    return sp.diags([np.full(n - 1, lo), np.full(n, d), np.full(n - 1, up)], [-1, 0, 1], format="csr")


def laplacian_1d(n: int) -> sp.csr_matrix:
    """tridiag(-1, 2, -1)."""
    return _tridiag(n, -1.0, 2.0, -1.0)


def laplacian_2d(nx: int, ny: int | None = None) -> sp.csr_matrix:
    """5-point Dirichlet Laplacian, unscaled: 4 on the diagonal, -1 off."""
    ny = nx if ny is None else ny
    A = sp.kron(sp.identity(ny), laplacian_1d(nx)) + sp.kron(laplacian_1d(ny), sp.identity(nx))
    A = A.tocsr()
    A.sort_indices()
    return A


def laplacian_3d(n1: int) -> sp.csr_matrix:
    """7-point Dirichlet Laplacian on n1^3, unscaled: 6 on the diagonal, -1 off."""
    T = laplacian_1d(n1)
    I = sp.identity(n1)
    A = sp.kron(I, sp.kron(I, T)) + sp.kron(I, sp.kron(T, I)) + sp.kron(T, sp.kron(I, I))
    A = A.tocsr()
    A.sort_indices()
    return A


def convdiff_2d(N: int, beta=(50.0, 25.0)) -> sp.csr_matrix:
    """-Lap u + beta . grad u on the unit square, N x N interior points,
    h = 1/(N+1), first-order upwind (beta > 0), scaled by h^-2 and h^-1."""
    h = 1.0 / (N + 1)
    bx, by = beta

    def dir_op(b):
        D2 = _tridiag(N, -1.0, 2.0, -1.0) / (h * h)
        D1 = _tridiag(N, -1.0, 1.0, 0.0) * (b / h)  # (u_i - u_{i-1}) / h
        return (D2 + D1).tocsr()

    A = sp.kron(sp.identity(N), dir_op(bx)) + sp.kron(dir_op(by), sp.identity(N))
    A = A.tocsr()
    A.sort_indices()
    return A


def laplacian_3d_bounds(n1: int):
    """Analytic extreme eigenvalues of the unscaled 7-point Laplacian on n1^3."""
    lam = lambda k: 4.0 * math.sin(math.pi * k / (2.0 * (n1 + 1))) ** 2
    return 3.0 * lam(1), 3.0 * lam(n1)


def grid_edges(N: int):
    """Edges of the N x N grid graph: horizontal ones first (row-major), then vertical."""
    idx = np.arange(N * N).reshape(N, N)
    hi, hj = idx[:, :-1].ravel(), idx[:, 1:].ravel()
    vi, vj = idx[:-1, :].ravel(), idx[1:, :].ravel()
    return np.concatenate([hi, vi]), np.concatenate([hj, vj])


def graph_laplacian(n: int, ei, ej, w, shift: float = 0.0) -> sp.csr_matrix:
    """L = sum_e w_e (e_i - e_j)(e_i - e_j)^T + shift * I."""
    W = sp.coo_matrix((np.concatenate([w, w]), (np.concatenate([ei, ej]), np.concatenate([ej, ei]))),
                      shape=(n, n)).tocsr()
    d = np.asarray(W.sum(axis=1)).ravel() + shift
    L = (sp.diags(d) - W).tocsr()
    L.sum_duplicates()
    L.sort_indices()
    return L


def rgg_knn_laplacian(n: int, k: int, rng: np.random.Generator, shift: float = 1e-3) -> sp.csr_matrix:
    """Random geometric graph in the unit square, k nearest neighbours,
    symmetrised (union, larger weight kept), weights lognormal(0, 0.5),
    graph Laplacian + shift * I."""
    from scipy.spatial import cKDTree

    pts = rng.random((n, 2))
    _, nb = cKDTree(pts).query(pts, k=k + 1)
    ei = np.repeat(np.arange(n), k)
    ej = nb[:, 1:].ravel()
    w = rng.lognormal(0.0, 0.5, size=ei.shape[0])
    W = sp.coo_matrix((w, (ei, ej)), shape=(n, n)).tocsr()
    W = W.maximum(W.T).tocoo()
    upper = W.row < W.col
    return graph_laplacian(n, W.row[upper], W.col[upper], W.data[upper], shift)


def read_matrix_market(path) -> sp.csr_matrix:
    """Coordinate real/integer/pattern MatrixMarket, general, symmetric or
    skew-symmetric, 1-based (the format of the reference's fixture
    examples/polynomial/laplacian.mtx, which stores the lower triangle of a
    symmetric matrix)."""
    with open(path) as f:
        header = f.readline().lower().split()
        if len(header) < 5 or header[0] != "%%matrixmarket" or header[2] != "coordinate":
            raise ValueError("only coordinate MatrixMarket files are supported")
        if header[3] not in ("real", "integer", "pattern"):
            raise ValueError(f"unsupported MatrixMarket field {header[3]!r} (real, integer or pattern)")
        if header[4] not in ("general", "symmetric", "skew-symmetric"):
            raise ValueError(f"unsupported MatrixMarket symmetry {header[4]!r}")
        symm = header[4] != "general"
        skew = header[4] == "skew-symmetric"
        line = f.readline()
        while line.startswith("%") or not line.strip():
            line = f.readline()
        nr, nc, nz = (int(t) for t in line.split())
        ncol = 2 if header[3] == "pattern" else 3
        data = np.loadtxt(f, ndmin=2, max_rows=nz) if nz > 0 else np.zeros((0, ncol))
    if data.shape[0] != nz or data.shape[1] < ncol:
        raise ValueError(f"expected {nz} entries of {ncol} columns, read {data.shape[0]}")
    i = data[:, 0].astype(np.int64) - 1
    j = data[:, 1].astype(np.int64) - 1
    if nz and (i.min() < 0 or j.min() < 0 or i.max() >= nr or j.max() >= nc):
        raise ValueError("MatrixMarket entry index out of range")
    v = data[:, 2].astype(np.float64) if ncol == 3 else np.ones(len(i))
    if symm:
        off = i != j
        i, j, v = (np.concatenate([i, j[off]]), np.concatenate([j, i[off]]),
                   np.concatenate([v, -v[off] if skew else v[off]]))
    A = sp.coo_matrix((v, (i, j)), shape=(nr, nc)).tocsr()
    A.sort_indices()
    return A


def unit(v: np.ndarray) -> np.ndarray:
    return v / np.linalg.norm(v)


@dataclass
class Problem:
    name: str
    A: sp.csr_matrix
    x: np.ndarray
    params: dict


def laplace2d_expm() -> Problem:
    A = laplacian_2d(100)
    x = unit(np.random.default_rng(0).uniform(-1.0, 1.0, A.shape[0]))
    return Problem("laplace2d-100x100 exp(-A)x m<=50 eps=1e-10", A, x,
                   dict(t=1.0, itmax=50, eps=1e-10))


def laplace3d_lanczos(n1: int = 128) -> Problem:
    A = laplacian_3d(n1)
    x = unit(np.random.default_rng(1).standard_normal(A.shape[0]))
    return Problem(f"laplace3d-{n1}^3 exp(-0.05A)x lanczos m=80", A, x, dict(t=0.05, m=80))


def convdiff_phi1(N: int = 2048) -> Problem:
    A = convdiff_2d(N)
    x = unit(np.random.default_rng(1).standard_normal(A.shape[0]))
    return Problem(f"convdiff2d-{N}^2 phi1(-1e-3A)x arnoldi m=60", A, x, dict(t=1e-3, m=60))


def laplace3d_invsqrt(n1: int = 96) -> Problem:
    A = laplacian_3d(n1)
    x = np.random.default_rng(2).standard_normal(A.shape[0])
    return Problem(f"laplace3d-{n1}^3 A^-1/2 x HHT N=24", A, x,
                   dict(N=24, bounds=laplacian_3d_bounds(n1), eps=1e-10))


def uneven_batch(count: int = 64, nrhs: int = 4, scale: float = 1.0):
    """64 uneven instances: 32 2-D Laplacians (side ~ U{64..512}) and 32 kNN
    random-geometric-graph Laplacians (n log-uniform in [4096, 262144]);
    `scale` < 1 shrinks the sizes for tests."""
    rng = np.random.default_rng(3)
    out = []
    for i in range(count):
        if i < count // 2:
            side = int(rng.integers(64, 513))
            side = max(8, int(side * math.sqrt(scale)))
            A = laplacian_2d(side)
            kind = f"lap2d-{side}"
        else:
            n = int(round(math.exp(rng.uniform(math.log(4096), math.log(262144)))))
            n = max(64, int(n * scale))
            A = rgg_knn_laplacian(n, 8, rng)
            kind = f"rgg-{n}"
        X = rng.standard_normal((nrhs, A.shape[0]))
        t = float(rng.uniform(0.01, 1.0))
        out.append(Problem(kind, A, X, dict(t=t, m=60, eps=1e-8)))
    return out


def uneven_spd_batch(count: int = 64, nrhs: int = 4):
    """64 uneven SPD instances for the quadrature batch: 32 2-D Laplacians
    (side ~ U{32..128}) and 32 kNN random-geometric-graph Laplacians + 0.05 I
    (n log-uniform in [1024, 16384]), each with its spectral bounds in
    params["bounds"] (analytic for the grids, [0.05, max row sum] for the
    graphs)."""
    rng = np.random.default_rng(13)
    out = []
    for i in range(count):
        if i < count // 2:
            side = int(rng.integers(32, 129))
            A = laplacian_2d(side)
            lam = lambda j: 4.0 * math.sin(math.pi * j / (2.0 * (side + 1))) ** 2
            bounds = [2.0 * lam(1), 2.0 * lam(side)]
            kind = f"lap2d-{side}"
        else:
            n = int(round(math.exp(rng.uniform(math.log(1024), math.log(16384)))))
            A = rgg_knn_laplacian(n, 8, rng, shift=0.05)
            bounds = [0.05, float(abs(A).sum(axis=1).max())]
            kind = f"rgg-{n}"
        X = rng.standard_normal((nrhs, A.shape[0]))
        out.append(Problem(kind, A, X, dict(bounds=bounds)))
    return out


def skewed_rows(n: int, alpha: float = 1.5, seed: int = 5, lmin: int = 4, lmax: int = 4000,
                integer: bool = False) -> sp.csr_matrix:
    """n x n matrix with power-law row lengths: len = min(lmax, floor(lmin u^(-1/alpha))),
    u ~ U(0,1], so P(len > L) = (lmin/L)^alpha (alpha 1.5: mean ~12, about 250
    rows per million longer than 1000); columns uniform without repetition in
    a row, values N(0,1) (or nonzero integers in [-3, 3], for exact sums)."""
    rng = np.random.default_rng(seed)
    u = 1.0 - rng.random(n)
    lens = np.minimum(lmax, np.floor(lmin * u ** (-1.0 / alpha))).astype(np.int64)
    lens = np.minimum(lens, n)
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lens, out=indptr[1:])
    nnz = int(indptr[-1])
    cols = rng.integers(0, n, size=nnz)
    A = sp.csr_matrix((np.ones(nnz), cols, indptr), shape=(n, n))
    A.sum_duplicates()  # a repeated column in a row merges
    A.sort_indices()
    if integer:
        v = rng.integers(1, 4, size=A.nnz) * rng.choice([-1.0, 1.0], size=A.nnz)
        A.data = v.astype(np.float64)
    else:
        A.data = rng.standard_normal(A.nnz)
    return A


def grid_graph_adjoint(N: int = 512):
    rng = np.random.default_rng(4)
    ei, ej = grid_edges(N)
    theta = rng.lognormal(0.0, 0.7, size=ei.shape[0])
    theta_star = rng.lognormal(0.0, 0.7, size=ei.shape[0])
    x = rng.standard_normal(N * N)
    return dict(N=N, ei=ei, ej=ej, theta=theta, theta_star=theta_star, x=x, t=0.1)
