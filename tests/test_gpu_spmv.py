"""CSR SpMV on the GPU: index handling is bit-exact (integer-valued data makes
every product and sum exact, so any indexing slip changes the result)."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def int_matrix(n, density, seed, long_rows=()):
    rng = np.random.default_rng(seed)
    if n <= 2000:
        A = sp.random(n, n, density=density, random_state=seed, format="coo")
        rows, cols = [A.row.astype(np.int64)], [A.col.astype(np.int64)]
    else:  # coordinates drawn directly (duplicates merge)
        k = int(density * n * n)
        rows, cols = [rng.integers(0, n, size=k)], [rng.integers(0, n, size=k)]
    for r in long_rows:
        c = rng.choice(n, size=min(n, 5000), replace=False)
        rows.append(np.full(len(c), r, dtype=np.int64))
        cols.append(c.astype(np.int64))
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    A = sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(n, n))
    A.data = rng.integers(-3, 4, size=A.nnz).astype(np.float64)
    A.eliminate_zeros()
    A.sort_indices()
    return A


# 600,000 rows: about 1,250 tiles, several per block of the pipeline (the
# producer's four stages wrap around), with long rows among them
@pytest.mark.parametrize("n,density,long_rows", [(1, 1.0, ()), (37, 0.2, ()), (5000, 0.002, ()),
                                                  (20000, 0.0004, (3, 19999)), (6000, 0.0, ()),
                                                  (600000, 8e-6, (0, 123457, 599999))])
def test_spmv_bit_exact(lib, n, density, long_rows):
    import psfun_gb300 as pg
    A = int_matrix(n, density, n, long_rows)
    x = np.random.default_rng(1).integers(-5, 6, size=n).astype(np.float64)
    a = pg.CsrMatrix.from_scipy(A)
    y = a.spmv(x)
    assert np.array_equal(y, A @ x)
    y0 = np.random.default_rng(2).integers(-5, 6, size=n).astype(np.float64)
    y2 = a.spmv(x, alpha=2.0, beta=-3.0, y=y0)
    assert np.array_equal(y2, 2.0 * (A @ x) - 3.0 * y0)


# power-law row lengths: rows far longer than their warp-mates are summed by
# the whole warp (every split threshold from 32 to 2048 taken somewhere)
@pytest.mark.parametrize("n,alpha,seed", [(3000, 1.1, 21), (200000, 1.5, 22), (50000, 0.8, 23)])
def test_spmv_skewed_rows_bit_exact(lib, n, alpha, seed):
    import psfun_gb300 as pg
    from psfun_gb300 import matrices
    A = matrices.skewed_rows(n, alpha=alpha, seed=seed, integer=True)
    x = np.random.default_rng(seed).integers(-5, 6, size=n).astype(np.float64)
    a = pg.CsrMatrix.from_scipy(A)
    assert np.array_equal(a.spmv(x), A @ x)
    y0 = np.random.default_rng(seed + 1).integers(-5, 6, size=n).astype(np.float64)
    assert np.array_equal(a.spmv(x, alpha=2.0, beta=-3.0, y=y0), 2.0 * (A @ x) - 3.0 * y0)


def test_spmv_skewed_rows_float_matches_oracle(lib, orc):
    import psfun_gb300 as pg
    from psfun_gb300 import matrices
    A = matrices.skewed_rows(40000, alpha=1.2, seed=24)
    x = np.random.default_rng(25).standard_normal(A.shape[0])
    y = pg.CsrMatrix.from_scipy(A).spmv(x, alpha=0.9)
    ref = orc.spmv(orc.Csr.from_scipy(A), x, alpha=0.9)
    # a warp-summed row adds its entries in another order: rounding only
    scale = 0.9 * (abs(A) @ np.abs(x))
    assert np.all(np.abs(y - ref) <= 1e-13 * scale + 1e-300)


def test_spmv_one_based_input(lib):
    import psfun_gb300 as pg
    A = int_matrix(3000, 0.003, 7)
    a1 = pg.CsrMatrix(A.indptr + 1, A.indices + 1, A.data, index_base=1)
    x = np.arange(3000, dtype=np.float64) % 7 - 3
    assert np.array_equal(a1.spmv(x), A @ x)


def test_spmv_float_matches_oracle(lib, orc):
    import psfun_gb300 as pg
    from psfun_gb300 import matrices
    A = matrices.convdiff_2d(64)
    x = np.random.default_rng(3).standard_normal(A.shape[0])
    y = pg.CsrMatrix.from_scipy(A).spmv(x, alpha=-0.7)
    ref = orc.spmv(orc.Csr.from_scipy(A), x, alpha=-0.7)
    assert np.linalg.norm(y - ref) <= 1e-14 * np.linalg.norm(ref)


def test_invalid_csr_rejected(lib):
    import psfun_gb300 as pg
    with pytest.raises(pg.PsfunError) as e:
        pg.CsrMatrix([0, 1, 2], [0, 2], [1.0, 1.0])  # column 2 out of range for n = 2
    assert e.value.info == 9003
    with pytest.raises(pg.PsfunError) as e:
        pg.CsrMatrix([0, 2, 1], [0, 1], [1.0, 1.0])  # rowptr not monotone
    assert e.value.info == 9003


def test_spmv_device_pointers(lib):
    torch = pytest.importorskip("torch")
    import psfun_gb300 as pg
    A = int_matrix(4000, 0.003, 11)
    x = np.random.default_rng(4).integers(-5, 6, size=4000).astype(np.float64)
    a = pg.CsrMatrix.from_scipy(A)
    xd = torch.tensor(x, device="cuda")
    yd = a.spmv(xd)
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), A @ x)
