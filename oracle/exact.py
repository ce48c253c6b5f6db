"""Exact FP64 evaluations of f(A)x for the grid operators of the benchmark
workloads, through their Kronecker-sum structure -- TEST INFRASTRUCTURE ONLY
(the parity checker of tests/ and the accuracy figures of bench.py).

These are independent of the Krylov restatement in psfun_oracle.c: they use no
Krylov space, only the 1-D operators the grid matrices are assembled from.

  laplacian_3d_apply   f(L) x for the unscaled 7-point Dirichlet Laplacian on
                       n1^3 (L = T (+) T (+) T, T = tridiag(-1, 2, -1)), through
                       the eigenbasis of T (the discrete sine transform): every
                       f, exactly up to the rounding of three dense 1-D
                       transforms per axis.
  convdiff_phi1        phi_1(-t A) x for the 2-D upwind convection-diffusion
                       operator A = I (x) T_x + T_y (x) I of matrices.convdiff_2d,
                       as (t A)^{-1} (x - exp(-t A) x): exp(-t A) x is
                       E_y X E_x^T with the dense 1-D exponentials, and the
                       solve with A is the Sylvester equation
                       T_y Y + Y T_x^T = R, done by Bartels-Stewart with the real
                       Schur form of T_x^T only (T_y stays tridiagonal, so each
                       column is a banded solve) and blocked GEMM updates.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sl


def laplacian_1d_spectrum(n1: int):
    """Eigenvalues and orthonormal eigenvectors (columns) of tridiag(-1, 2, -1)."""
    k = np.arange(1, n1 + 1)
    lam = 4.0 * np.sin(np.pi * k / (2.0 * (n1 + 1))) ** 2
    Q = np.sqrt(2.0 / (n1 + 1)) * np.sin(np.outer(k, k) * np.pi / (n1 + 1))
    return lam, Q


def laplacian_3d_apply(n1: int, x, fun):
    """fun(L) x for the n1^3 7-point Laplacian; fun acts elementwise on the
    array of eigenvalues lam_i + lam_j + lam_k."""
    lam, Q = laplacian_1d_spectrum(n1)
    X = np.asarray(x, dtype=np.float64).reshape(n1, n1, n1)
    Xh = np.einsum("ia,jb,kc,ijk->abc", Q, Q, Q, X, optimize=True)
    L = lam[:, None, None] + lam[None, :, None] + lam[None, None, :]
    return np.einsum("ia,jb,kc,abc->ijk", Q, Q, Q, fun(L) * Xh, optimize=True).ravel()


def convdiff_1d(N: int, b: float) -> np.ndarray:
    """The dense 1-D factor of matrices.convdiff_2d: tridiag(-1, 2, -1)/h^2 +
    tridiag(-1, 1, 0) b/h with h = 1/(N+1)."""
    h = 1.0 / (N + 1)
    T = np.zeros((N, N))
    i = np.arange(N)
    T[i, i] = 2.0 / (h * h) + b / h
    T[i[1:], i[:-1]] = -1.0 / (h * h) - b / h
    T[i[:-1], i[1:]] = -1.0 / (h * h)
    return T


def sylvester_tridiag(Ty: np.ndarray, Tx: np.ndarray, R: np.ndarray, block: int = 64) -> np.ndarray:
    """Y with Ty Y + Y Tx^T = R, Ty tridiagonal (dense storage), by
    Bartels-Stewart on the real Schur form Tx^T = Q U Q^T: with Z = Y Q the
    columns satisfy (Ty + U_jj I) z_j = (R Q)_j - sum_{k<j} U_kj z_k, solved in
    order as banded systems, the coupling to earlier column blocks applied as
    one GEMM per block.  Requires the real Schur form to be triangular (real
    eigenvalues, true for the upwind operators)."""
    N = Ty.shape[0]
    U, Q = sl.schur(Tx.T, output="real")
    if np.any(np.diag(U, -1) != 0.0):
        raise ValueError("Tx has complex eigenvalues; the column recurrence needs a triangular Schur form")
    Rq = R @ Q
    ab = np.zeros((3, N))
    ab[0, 1:] = np.diag(Ty, 1)
    ab[2, :-1] = np.diag(Ty, -1)
    dy = np.diag(Ty).copy()
    Z = np.zeros_like(Rq)
    for j0 in range(0, N, block):
        j1 = min(N, j0 + block)
        B = Rq[:, j0:j1] - Z[:, :j0] @ U[:j0, j0:j1] if j0 else Rq[:, j0:j1].copy()
        for j in range(j0, j1):
            rhs = B[:, j - j0] - Z[:, j0:j] @ U[j0:j, j] if j > j0 else B[:, 0]
            ab[1] = dy + U[j, j]
            Z[:, j] = sl.solve_banded((1, 1), ab, rhs, check_finite=False)
    return Z @ Q.T


def convdiff_phi1(N: int, x, t: float, beta=(50.0, 25.0)) -> np.ndarray:
    """phi_1(-t A) x for A = matrices.convdiff_2d(N, beta) (row-major grid,
    index iy * N + ix): A vec(X) = T_y X + X T_x^T.  phi_1(M) = M^{-1}(e^M - I)
    with M = -t A gives y = (t A)^{-1} (x - exp(-t A) x)."""
    Tx, Ty = convdiff_1d(N, beta[0]), convdiff_1d(N, beta[1])
    X = np.asarray(x, dtype=np.float64).reshape(N, N)
    EX = sl.expm(-t * Ty) @ X @ sl.expm(-t * Tx).T
    Y = sylvester_tridiag(Ty, Tx, X - EX) / t
    return Y.ravel()
