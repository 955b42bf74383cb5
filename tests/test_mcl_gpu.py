"""GPU MCL expansion + prune/select against the reference's own output."""
import numpy as np
import pytest

from combblas_gb300 import generators as G
from combblas_gb300 import local
from combblas_gb300 import mcl
from conftest import golden_matrix

pytestmark = pytest.mark.gpu


def test_mcl_golden(gpu_ctx, oracle_lib, golden):
    O = oracle_lib
    M = golden_matrix(golden, "mcl4096")
    for thr, k in ((1e-4, 30), (1e-3, 12)):
        R, _ = mcl.mcl_expand(M, thr, k)
        cp, rows, vals = R.to_csc()
        key = f"mcl/mcl4096/{thr:g}/{k}"
        ecp, erows, evals = O.tuples_to_csc(golden[f"{key}/rows"], golden[f"{key}/cols"], golden[f"{key}/vals"],
                                            M.ncol)
        assert np.array_equal(cp, ecp) and np.array_equal(rows, erows) and np.array_equal(vals, evals)


def test_mcl_select_vs_oracle_ties_and_thresholds(gpu_ctx, oracle_lib):
    """Hand-made values with ties at the k-th value and entries exactly at
    the threshold (kept: the final prune removes only values < cut)."""
    O = oracle_lib
    rng = np.random.default_rng(2)
    n = 300
    cols, rows, vals = [], [], []
    for j in range(n):
        cnt = rng.integers(0, 60)
        r = np.sort(rng.choice(500, cnt, replace=False))
        v = rng.choice(np.array([1e-5, 1e-4, 2e-4, 0.01, 0.01, 0.02, 0.5], np.float32), cnt)
        cols.append(np.full(cnt, j))
        rows.append(r)
        vals.append(v)
    M = G.csc_from_coo(500, n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals).astype(np.float32))
    M.values = M.values.astype(np.float32)
    R = local.spgemm(G.CSC(500, 500, np.arange(501), np.arange(500), np.ones(500, np.float32)), M,
                     dtype=np.float32)  # identity * M on the GPU
    for thr, k in ((1e-4, 5), (1e-4, 1), (2e-4, 20), (0.0, 3)):
        S = mcl.MCLPruneRecoverySelect(R, thr, k)
        cp, rows_, vals_ = S.to_csc()
        ecp, erows, evals = O.port_mcl_select(M.colptr, M.rowidx, M.values, thr, k)
        assert np.array_equal(cp, ecp) and np.array_equal(rows_, erows) and np.array_equal(vals_, evals), (thr, k)


@pytest.mark.parametrize("n,cluster", [(1 << 14, 256), (1 << 16, 1024)])
def test_mcl_planted_vs_oracle(gpu_ctx, oracle_lib, n, cluster):
    O = oracle_lib
    M = G.mcl_planted(n, cluster, 24, 6, seed=n)
    R, _ = mcl.mcl_expand(M, 1e-4, 100)
    cp, rows, vals = R.to_csc()
    pcp, prow, pval = O.port_spgemm(M, M, O.SR_PLUSTIMES_F32, sorted=False)
    scp, srow, sval = O.port_mcl_select(pcp, prow, pval, 1e-4, 100)
    scp, srow, sval = O.canonical_csc(scp, srow, sval)
    assert np.array_equal(cp, scp) and np.array_equal(rows, srow) and np.array_equal(vals, sval)
