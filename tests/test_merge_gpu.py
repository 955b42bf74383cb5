"""MultiwayMerge on the GPU (the stacked-identity product) against the
reference's golden merges and the oracle's restatement."""
import numpy as np
import pytest

from combblas_gb300 import generators as G
from combblas_gb300 import local
from test_oracle import check_csc, merge_lists, typed

pytestmark = pytest.mark.gpu


def test_merge_golden(gpu_ctx, oracle_lib, golden):
    """Under the ordered fold the lists are folded in list order (the
    oracle's restatement); the exact fold is checked in the next test."""
    O = oracle_lib
    with gpu_ctx.folding("ordered"):
        _merge_golden(O, golden)


def _merge_golden(O, golden):
    for K in (2, 4):
        for sr, name, dt in ((O.SR_PLUSTIMES_F64, "plustimes", np.float64), (O.SR_SELECT2NDMIN_I64, "select2ndmin",
                                                                             np.int64)):
            lists = merge_lists(golden, K, sr, O)
            cp, rows, vals = local.MultiwayMerge(lists, 400, 250, sr=name, dtype=dt).to_csc()
            check_csc(cp, rows, vals, golden, f"merge/{K}/{sr}", sr, O.V_HYBRID, 250, O,
                      exact_values=(K == 2 or sr != O.SR_PLUSTIMES_F64))
            pcp, prow, pval = O.port_multiway_merge(lists, 400, 250, sr)
            assert np.array_equal(cp, pcp) and np.array_equal(rows, prow) and np.array_equal(vals, pval)


@pytest.mark.parametrize("sr", [0, 1, 2, 3, 4, 5, 6])
def test_merge_semirings_and_dcsc(gpu_ctx, oracle_lib, sr):
    O = oracle_lib
    from test_spgemm_gpu import SR_NAME

    name, dt = SR_NAME[sr]
    lists = [typed(G.random_sparse(700, 500, 0.01, seed=60 + k, empty_cols=0.3), sr, 70 + k, O) for k in range(3)]
    ins = [local.DCSC.from_csc(M) if k % 2 else M for k, M in enumerate(lists)]  # mixed CSC / DCSC inputs
    pcp, prow, pval = O.port_multiway_merge(lists, 700, 500, sr)
    with gpu_ctx.folding("ordered"):
        cp, rows, vals = local.MultiwayMerge(ins, 700, 500, sr=name, dtype=dt).to_csc()
    assert np.array_equal(cp, pcp) and np.array_equal(rows, prow) and np.array_equal(vals, pval)
    # the default exact fold: fp64 sums of three lists rounded once (within
    # the list-order fold's rounding); every other semiring unchanged
    cp, rows, vals = local.MultiwayMerge(ins, 700, 500, sr=name, dtype=dt).to_csc()
    assert np.array_equal(cp, pcp) and np.array_equal(rows, prow)
    if sr == 0:
        assert np.max(np.abs(vals - pval) / np.abs(pval)) <= 1e-15
    else:
        assert np.array_equal(vals, pval)


def test_merge_edges(gpu_ctx):
    from combblas_gb300._lib import GbcError

    R = local.MultiwayMerge([], 30, 20)
    assert R.nnz == 0 and R.nrow == 30 and R.ncol == 20
    A = G.random_sparse(30, 20, 0.2, seed=1)
    cp, rows, vals = local.MultiwayMerge([A], 30, 20).to_csc()
    assert np.array_equal(cp, A.colptr) and np.array_equal(rows, A.rowidx) and np.array_equal(vals, A.values)
    with pytest.raises(GbcError, match="dimensions"):
        local.MultiwayMerge([A, G.random_sparse(30, 21, 0.2, seed=2)], 30, 20)
