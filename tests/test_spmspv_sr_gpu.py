"""The other SpMXSpV semirings on the GPU (gbc_spmspv): Select2nd (the
boolean optbuf path of TopDownBFS), SelectMax, PlusTimes and SelectMin on
rectangular CSC / DCSC matrices, against the reference's own output and the
restatement, bit for bit."""
import ctypes

import numpy as np
import pytest

from combblas_gb300 import bfs as B
from combblas_gb300 import generators as G
from combblas_gb300 import _lib as L
from combblas_gb300.local import DCSC
from conftest import golden_matrix

pytestmark = pytest.mark.gpu

NAMES = {1: "select2nd", 2: "selectmax"}


def test_spmspv_semirings_golden(gpu_ctx, oracle_lib, golden):
    O = oracle_lib
    R = golden_matrix(golden, "rect1500")
    x = golden["spmspvsr/x_ind"]
    P = B.SpMSpVPlan(R)
    for sx, name in NAMES.items():
        r, v = P.multiply(x, golden["spmspvsr/x_i64"], name)
        assert np.array_equal(r, golden[f"spmspvsr/{sx}/y_ind"]) and np.array_equal(v, golden[f"spmspvsr/{sx}/y_val"])
    for dt in (np.float64, np.float32):
        name = np.dtype(dt).name
        Pd = B.SpMSpVPlan(R.with_values(R.values.astype(dt)), dt)
        r, v = Pd.multiply(x, golden["spmspvsr/x_f64"].astype(dt), "plustimes")
        assert np.array_equal(r, golden[f"spmspvsr/3/{name}/y_ind"])
        assert np.array_equal(v, golden[f"spmspvsr/3/{name}/y_val"]), name
    Pi = B.SpMSpVPlan(R.with_values(np.round(R.values * 100).astype(np.int64)), np.int64)
    r, v = Pi.multiply(x, golden["spmspvsr/x_i64"], "plustimes")
    assert np.array_equal(r, golden["spmspvsr/3/int64/y_ind"]) and np.array_equal(v, golden["spmspvsr/3/int64/y_val"])


@pytest.mark.parametrize("scale", [12, 16])
def test_spmspv_semirings_rmat_vs_port(gpu_ctx, oracle_lib, scale):
    """R-MAT pattern (hub rows up to thousands of hits) and uneven frontiers."""
    O = oracle_lib
    A = G.rmat(scale, 16, seed=scale)
    rng = np.random.default_rng(scale)
    n = A.ncol
    Pp = B.SpMSpVPlan(A)
    Pf = B.SpMSpVPlan(A, np.float64)
    for nx in (1, 37, n // 16, n // 2):
        x = np.sort(rng.choice(n, nx, replace=False)).astype(np.int32)
        xi = rng.integers(-(1 << 40), 1 << 40, nx)
        for sx, name in ((0, "selectmin"), (1, "select2nd"), (2, "selectmax")):
            r, v = Pp.multiply(x, xi, name)
            if sx == 0:
                er, ev = O.port_spmspv(A.with_values(None), x, xi)
            else:
                er, ev = O.port_spmspv_sr(A, sx, x, xi)
            assert np.array_equal(r, er) and np.array_equal(v, ev), (name, nx)
        xf = rng.random(nx) * 2 - 1
        r, v = Pf.multiply(x, xf, "plustimes")
        er, ev = O.port_spmspv_sr(A, O.SX_PLUSTIMES, x, xf, np.float64)
        assert np.array_equal(r, er) and np.array_equal(v, ev), ("plustimes", nx)


def test_spmspv_dcsc_rectangular_and_repeat(gpu_ctx, oracle_lib):
    """A DCSC operand with empty columns, wider than tall; the plan serves
    repeated calls (the scratch returns to its initial state) and its
    matrix is copied to the device once."""
    O = oracle_lib
    rng = np.random.default_rng(5)
    m, n = 700, 5000
    cols = rng.choice(n, 400, replace=False)
    A = G.csc_from_coo(m, n, rng.integers(0, m, 6000), rng.choice(cols, 6000), rng.random(6000))
    D = DCSC.from_csc(A)
    P = B.SpMSpVPlan(D, np.float64)
    info = [ctypes.c_int64() for _ in range(3)]
    L.check(L.lib().gbc_spmspv_plan_info(P.h, *[ctypes.byref(i) for i in info]))
    assert [i.value for i in info] == [m, n, A.nnz]
    x = np.sort(rng.choice(n, 900, replace=False)).astype(np.int32)
    xf = rng.random(900)
    first = P.multiply(x, xf, "plustimes")
    for _ in range(3):
        again = P.multiply(x, xf, "plustimes")
        assert all(np.array_equal(a, b) for a, b in zip(first, again))
    er, ev = O.port_spmspv_sr(A, O.SX_PLUSTIMES, x, xf, np.float64)
    assert np.array_equal(first[0], er) and np.array_equal(first[1], ev)
    xi = rng.integers(0, 1000, 900)
    r, v = P.multiply(x, xi, "select2nd")
    er, ev = O.port_spmspv_sr(A, O.SX_SELECT2ND, x, xi)
    assert np.array_equal(r, er) and np.array_equal(v, ev)
    r, v = P.multiply(np.zeros(0, np.int32), np.zeros(0), "plustimes")
    assert len(r) == 0


def test_spmspv_bad_vectors(gpu_ctx):
    A = G.rmat(8, 8, seed=1)
    P = B.SpMSpVPlan(A)
    with pytest.raises(RuntimeError, match="repeated"):
        P.multiply(np.array([3, 3], np.int32), np.array([1, 2]), "select2nd")
    with pytest.raises(RuntimeError, match="out of range"):
        P.multiply(np.array([1, A.ncol], np.int32), np.array([1, 2]), "selectmax")
    with pytest.raises(RuntimeError):
        P.multiply(np.array([1], np.int32), np.array([1.0]), "plustimes")  # pattern plan
    # the plan still works after the rejected calls
    r, v = P.multiply(np.array([0, 5], np.int32), np.array([7, 9]), "selectmax")
    assert len(r) == len(set(r.tolist()))
