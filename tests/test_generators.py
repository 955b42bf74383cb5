import numpy as np

from combblas_gb300 import generators as G


def test_rmat_symmetric_no_loops_sorted():
    A = G.rmat(10, 8, seed=3)
    d = A.to_dense() != 0
    assert (d == d.T).all()
    assert not d.diagonal().any()
    for j in range(A.ncol):
        r = A.rowidx[A.colptr[j]:A.colptr[j + 1]]
        assert (np.diff(r) > 0).all()
    assert ((A.values > 0) & (A.values <= 1)).all()


def test_rmat_seeded():
    a = G.rmat(9, 4, seed=7)
    b = G.rmat(9, 4, seed=7)
    assert np.array_equal(a.rowidx, b.rowidx) and np.array_equal(a.values, b.values)


def test_mcl_column_stochastic():
    M = G.mcl_planted(2048, 128, 8, 2, seed=1)
    s = np.add.reduceat(M.values.astype(np.float64), M.colptr[:-1])
    assert np.allclose(s, 1.0, atol=1e-5)
    assert (np.diff(M.colptr) >= 1).all()


def test_poisson_and_aggregation():
    A = G.poisson27(4)
    d = A.to_dense()
    assert (np.diag(d) == 26).all() and (d == d.T).all()
    R = G.aggregation(4)
    assert R.nrow == 8 and R.ncol == 64 and R.nnz == 64
