"""The MatrixMarket reader (the input format of the reference's drivers,
examples/polynomial/laplacian.mtx read through psb_mat_read) against scipy's
writer: general, symmetric, skew-symmetric, integer and pattern files, an
empty matrix, and the errors for unsupported files."""

import numpy as np
import pytest
import scipy.io
import scipy.sparse as sp

from psfun_gb300 import matrices


def roundtrip(tmp_path, A, **kw):
    path = tmp_path / "a.mtx"
    scipy.io.mmwrite(str(path), A, **kw)
    return matrices.read_matrix_market(path)


def test_general(tmp_path):
    A = sp.random(40, 30, density=0.1, random_state=1, format="csr")
    B = roundtrip(tmp_path, A)
    assert B.shape == A.shape and B.has_sorted_indices
    assert abs(B - A).max() == 0.0


def test_symmetric_lower_triangle(tmp_path):
    """The fixture's layout: only the lower triangle is stored."""
    T = -matrices.laplacian_1d(50)
    path = tmp_path / "t.mtx"
    scipy.io.mmwrite(str(path), T, symmetry="symmetric")
    body = path.read_text().splitlines()
    assert "symmetric" in body[0]
    B = matrices.read_matrix_market(path)
    assert B.nnz == 148 and abs(B - T).max() == 0.0


def test_skew_symmetric(tmp_path):
    R = sp.random(20, 20, density=0.2, random_state=2)
    S = (R - R.T).tocsr()
    S.eliminate_zeros()
    B = roundtrip(tmp_path, S, symmetry="skew-symmetric")
    assert abs(B - S).max() == 0.0


def test_integer_and_pattern(tmp_path):
    A = sp.csr_matrix(np.array([[0, 3, 0], [-2, 0, 0], [0, 0, 7]]))
    B = roundtrip(tmp_path, A, field="integer")
    assert B.dtype == np.float64 and abs(B - A).max() == 0.0
    P = roundtrip(tmp_path, A, field="pattern")
    assert abs(P - (A != 0).astype(np.float64)).max() == 0.0


def test_comments_and_empty(tmp_path):
    path = tmp_path / "e.mtx"
    path.write_text("%%MatrixMarket matrix coordinate real general\n% a comment\n\n4 5 0\n")
    B = matrices.read_matrix_market(path)
    assert B.shape == (4, 5) and B.nnz == 0


@pytest.mark.parametrize("text,msg", [
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", "coordinate"),
    ("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1.0 2.0\n", "field"),
    ("%%MatrixMarket matrix coordinate real hermitian\n1 1 1\n1 1 1.0\n", "symmetry"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n", "expected 2 entries"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n", "out of range"),
])
def test_rejects(tmp_path, text, msg):
    path = tmp_path / "bad.mtx"
    path.write_text(text)
    with pytest.raises(ValueError, match=msg):
        matrices.read_matrix_market(path)
