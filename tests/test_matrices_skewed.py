"""The power-law row-length generator behind the SpMV row-splitting tests and
`bench.py --only skewed`: deterministic per seed, CSR with sorted unique
columns, lengths within [lmin, lmax] (a repeated column in a row merges, so
a row may come out shorter, never longer), the tail the power law promises,
and integer values for exact sums.  CPU only."""
import numpy as np

from psfun_gb300 import matrices


def test_skewed_rows_shape_and_determinism():
    A = matrices.skewed_rows(20000, alpha=1.5, seed=9)
    B = matrices.skewed_rows(20000, alpha=1.5, seed=9)
    assert A.shape == (20000, 20000) and A.has_sorted_indices
    assert np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)
    assert np.array_equal(A.data, B.data)
    lens = np.diff(A.indptr)
    assert lens.max() <= 4000 and lens.min() >= 1
    for r in range(0, 20000, 997):  # no repeated column within a row
        cols = A.indices[A.indptr[r]:A.indptr[r + 1]]
        assert np.all(np.diff(cols) > 0)


def test_skewed_rows_tail():
    # P(len > L) = (4 / L)^alpha before merging: at alpha 1.5 and n = 2^20 the
    # rows above 1000 entries number about 262 and the mean length is ~11
    n = 1 << 20
    A = matrices.skewed_rows(n, alpha=1.5, seed=5)
    lens = np.diff(A.indptr)
    assert 200 <= int((lens > 1000).sum()) <= 330
    assert 9.0 <= lens.mean() <= 13.5
    assert int((lens > 32).sum()) > 0.005 * n


def test_skewed_rows_integer_values():
    A = matrices.skewed_rows(5000, seed=3, integer=True)
    v = np.unique(A.data)
    assert set(v.tolist()) <= {-3.0, -2.0, -1.0, 1.0, 2.0, 3.0}
