"""COO -> CSR / ELL with the (row, column) ordering sorted on the GPU, and
COO -> DENSE scattered on the GPU (tbsla_matrix_convert_device,
kernels/sort.cu): the arrays equal the host conversion's exactly -- the host
conversion itself is pinned to the reference's converting constructors by
the golden tests -- including duplicate (row, column) pairs, which keep
their storage order (DENSE: summed in that order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def coo_of(T, n_row, n_col, row, col, val):
    return T.MatrixCOO.from_arrays(n_row, n_col, np.asarray(row, np.int32), np.asarray(col, np.int32),
                                   np.asarray(val, np.float64))


def same(a, b):
    ia, ib = a.info(), b.info()
    assert ia == ib
    xa, xb = a.arrays(), b.arrays()
    assert xa.keys() == xb.keys()
    for k in xa:
        assert np.array_equal(xa[k], xb[k]), k


@pytest.mark.parametrize("shape", [(1, 1, 1), (17, 5, 60), (1000, 3000, 20000), (70000, 70000, 1_000_000),
                                   (3, 1 << 30, 50)])
def test_device_order_equals_host(gpu, shape):
    T = gpu
    n_row, n_col, nnz = shape
    rng = np.random.default_rng(n_row + nnz)
    row = rng.integers(0, n_row, nnz)
    col = rng.integers(0, min(n_col, 1 << 20) if n_col > (1 << 20) else n_col, nnz)
    if n_col > (1 << 20):
        col = col + (n_col - (1 << 20))  # high column bits in use
    # duplicates: repeat a slice of the entries with other values
    k = nnz // 10
    row = np.concatenate([row, row[:k]])
    col = np.concatenate([col, col[:k]])
    val = rng.uniform(-1, 1, len(row))
    coo = coo_of(T, n_row, n_col, row, col, val)
    for cls in (T.MatrixCSR, T.MatrixELL):
        same(cls(coo), cls(coo, device=True))
    if n_row * n_col <= (1 << 27):
        same(T.MatrixDENSE(coo), T.MatrixDENSE(coo, device=True))


def test_device_order_power_law_and_empty(gpu):
    T = gpu
    n = 1 << 17
    m = T.MatrixCSR()
    m.fill_powerlaw(n, seed=4)
    a = m.arrays()
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(a["rowptr"]))
    perm = np.random.default_rng(1).permutation(len(rows))
    coo = coo_of(T, n, n, rows[perm], a["colidx"][perm], a["values"][perm])
    d = T.MatrixCSR(coo, device=True)
    same(T.MatrixCSR(coo), d)
    # sorted columns within rows and the same entries as the generator's CSR
    same(m, d)
    empty = coo_of(T, 5, 5, [], [], [])
    same(T.MatrixCSR(empty), T.MatrixCSR(empty, device=True))


def test_device_dense_scatter_duplicates_and_cdiag(gpu):
    """Many duplicates of a few positions, summed in storage order exactly as
    MatrixDENSE(const MatrixCOO&) does; and the reference's cdiag matrix."""
    T = gpu
    rng = np.random.default_rng(9)
    row = rng.integers(0, 7, 5000)
    col = rng.integers(0, 5, 5000)
    val = rng.uniform(-1, 1, 5000) * 10.0 ** rng.integers(-8, 8, 5000)
    coo = coo_of(T, 7, 5, row, col, val)
    same(T.MatrixDENSE(coo), T.MatrixDENSE(coo, device=True))
    c = T.MatrixCOO()
    c.fill_cdiag(300, 200, 3)
    same(T.MatrixDENSE(c), T.MatrixDENSE(c, device=True))
