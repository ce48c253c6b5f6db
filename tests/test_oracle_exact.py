"""The Kronecker-structure exact evaluations of oracle/exact.py against dense
SciPy evaluations on small grids (CPU)."""
import numpy as np
import scipy.linalg as sl

from oracle import exact
from psfun_gb300 import matrices


def test_laplacian_3d_apply_equals_dense_expm():
    n1 = 6
    A = matrices.laplacian_3d(n1).toarray()
    x = np.random.default_rng(0).standard_normal(n1 ** 3)
    y = exact.laplacian_3d_apply(n1, x, lambda L: np.exp(-0.3 * L))
    ref = sl.expm(-0.3 * A) @ x
    assert np.linalg.norm(y - ref) <= 1e-14 * np.linalg.norm(ref)


def test_convdiff_factors_assemble_the_operator():
    N = 9
    A = matrices.convdiff_2d(N).toarray()
    Tx, Ty = exact.convdiff_1d(N, 50.0), exact.convdiff_1d(N, 25.0)
    assert np.array_equal(A, np.kron(np.eye(N), Tx) + np.kron(Ty, np.eye(N)))


def test_sylvester_tridiag_equals_scipy():
    N = 120
    Tx, Ty = exact.convdiff_1d(N, 50.0), exact.convdiff_1d(N, 25.0)
    R = np.random.default_rng(1).standard_normal((N, N))
    Y = exact.sylvester_tridiag(Ty, Tx, R, block=16)
    ref = sl.solve_sylvester(Ty, Tx.T, R)
    assert np.linalg.norm(Y - ref) <= 1e-11 * np.linalg.norm(ref)


def test_convdiff_phi1_equals_augmented_expm():
    for N in (16, 30):
        t = 1e-3
        x = matrices.unit(np.random.default_rng(N).standard_normal(N * N))
        y = exact.convdiff_phi1(N, x, t)
        n = N * N
        aug = np.zeros((n + 1, n + 1))
        aug[:n, :n] = -t * matrices.convdiff_2d(N).toarray()
        aug[:n, n] = x
        ref = sl.expm(aug)[:n, n]
        assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)
