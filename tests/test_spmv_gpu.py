"""Dense-vector SpMV (dcsc_gespmv) on the GPU against the reference's golden
results and the oracle's restatement."""
import numpy as np
import pytest

from combblas_gb300 import generators as G
from combblas_gb300 import local
from conftest import golden_matrix
from test_oracle import typed

pytestmark = pytest.mark.gpu

NAME = {0: "plustimes", 1: "plustimes", 2: "plustimes", 3: "minplus", 4: "select2ndmin", 5: "bool", 6: "minplus"}


def check(sr, y, ref, O):
    if sr in (O.SR_PLUSTIMES_F64, O.SR_PLUSTIMES_F32):
        tol = 1e-12 if sr == O.SR_PLUSTIMES_F64 else 1e-5  # fixed row order vs the reference's column order
        rel = np.abs(y - ref) / np.maximum(np.abs(ref), np.finfo(ref.dtype).tiny)
        assert rel.max(initial=0) <= tol, rel.max()
    else:
        assert np.array_equal(y, ref)


def test_spmv_golden(gpu_ctx, oracle_lib, golden):
    O = oracle_lib
    M = golden_matrix(golden, "rmat8")
    for sr in (O.SR_PLUSTIMES_F64, O.SR_MINPLUS_F64, O.SR_SELECT2NDMIN_I64, O.SR_BOOL):
        A = typed(M, sr, 50 + sr, O)
        y = np.array(golden[f"spmv/{sr}/y0"])
        local.dcsc_gespmv(A, golden[f"spmv/{sr}/x"], y, sr=NAME[sr])
        check(sr, y, golden[f"spmv/{sr}/y"], O)


def vectors(sr, m, n, O, seed):
    rng = np.random.default_rng(seed)
    dt = O.SR_DTYPE[sr]
    if dt == np.bool_:
        return rng.random(n) < 0.5, rng.random(m) < 0.2
    if dt == np.int64:
        return rng.integers(0, 100, n), rng.integers(0, 1000, m)
    return rng.random(n).astype(dt), (rng.random(m) * 3).astype(dt)


@pytest.mark.parametrize("sr", [0, 1, 2, 3, 4, 5, 6])
def test_spmv_rmat_vs_oracle(gpu_ctx, oracle_lib, sr):
    O = oracle_lib
    A = typed(G.rmat(12, 8, seed=7), sr, 80 + sr, O)
    x, y0 = vectors(sr, A.nrow, A.ncol, O, 9)
    plan = local.SpMVPlan(A, O.SR_DTYPE[sr])
    y = plan.multiply(x, np.array(y0), NAME[sr])
    check(sr, y, O.port_spmv(A, x, y0, sr), O)
    y2 = plan.multiply(x, np.array(y0), NAME[sr])
    assert np.array_equal(y, y2)  # repeated runs are bit-identical
    plan.close()


def test_spmv_rectangular_dcsc_device(gpu_ctx, oracle_lib):
    """Tall rectangular DCSC input with empty rows and columns; device x/y."""
    import torch

    O = oracle_lib
    A = G.random_sparse(5000, 700, 0.002, seed=4, empty_cols=0.3)
    x, y0 = vectors(0, A.nrow, A.ncol, O, 3)
    plan = local.SpMVPlan(local.DCSC.from_csc(A))
    dx = torch.from_numpy(x).cuda()
    dy = torch.from_numpy(np.array(y0)).cuda()
    plan.multiply(dx.data_ptr(), dy.data_ptr())
    ref = O.port_spmv(A, x, y0, 0)
    check(0, dy.cpu().numpy(), ref, O)
    empty = np.bincount(A.rowidx, minlength=A.nrow) == 0
    assert np.array_equal(dy.cpu().numpy()[empty], y0[empty])  # rows without entries keep y
    plan.close()
