"""Batched uneven SpGEMMs (one launch per pass, CUDA-graph replay) against
the same products computed one by one and against the oracle."""
import numpy as np
import pytest

from combblas_gb300 import batch as BT
from combblas_gb300 import generators as G
from combblas_gb300 import local

pytestmark = pytest.mark.gpu


def small_c4():
    rm, gk = G.batch_c4(nprob=12, seed=9, rmat_scales=(6, 12), sides=(4, 10))
    return rm, gk


def test_batch_matches_one_by_one_and_oracle(gpu_ctx, oracle_lib):
    O = oracle_lib
    rm, gk = small_c4()
    As = rm + [A for A, R, Rt in gk]
    Bs = rm + [Rt for A, R, Rt in gk]
    b = BT.Batch(As, Bs)
    b.run()  # a replay of the captured graph recomputes everything
    for p, (A, B) in enumerate(zip(As, Bs)):
        cp, ir, num = b.result(p)
        ecp, eir, enum = local.spgemm(A, B).to_csc()
        assert np.array_equal(cp, ecp) and np.array_equal(ir, eir) and np.array_equal(num, enum), p
        pcp, pir, pnum = O.port_spgemm(A, B, O.SR_PLUSTIMES_F64, fold="exact")  # the default fold
        assert np.array_equal(cp, pcp) and np.array_equal(ir, pir) and np.array_equal(num, pnum), p
    b.close()


def test_galerkin_two_stage_batch(gpu_ctx, oracle_lib):
    """R * (A * R^T) as two batches, the second fed from the first's device
    results; Galerkin values are small integers, so they are exact."""
    O = oracle_lib
    _, gk = small_c4()
    b1 = BT.Batch([A for A, R, Rt in gk], [Rt for A, R, Rt in gk])
    ARs = [b1.result_device(p, A.nrow, Rt.ncol) for p, (A, R, Rt) in enumerate(gk)]
    b2 = BT.Batch([R for A, R, Rt in gk], ARs)
    for p, (A, R, Rt) in enumerate(gk):
        cp, ir, num = b2.result(p)
        pcp, pir, pnum = O.port_spgemm(A, Rt, O.SR_PLUSTIMES_F64)
        AR = G.CSC(A.nrow, Rt.ncol, pcp, pir, pnum)
        qcp, qir, qnum = O.port_spgemm(R, AR, O.SR_PLUSTIMES_F64)
        assert np.array_equal(cp, qcp) and np.array_equal(ir, qir) and np.array_equal(num, qnum)
        assert np.all(num == np.round(num))
    b2.close()
    b1.close()


@pytest.mark.parametrize("s1,s2", [(0, 0), (64, 1024), (256, 4096)])
def test_thresholds_do_not_change_results(gpu_ctx, s1, s2):
    rm, _ = small_c4()
    b0 = BT.Batch(rm, rm, s1=256, s2=4096)
    b = BT.Batch(rm, rm, s1=s1, s2=s2)
    for p in range(len(rm)):
        assert all(np.array_equal(x, y) for x, y in zip(b0.result(p), b.result(p)))
    b.close()
    b0.close()


def test_autotuner_caches_choice(gpu_ctx, tmp_path):
    rm, _ = small_c4()
    cache = str(tmp_path / "tune.json")
    choice, timings = BT.autotune(rm, rm, cache=cache, reps=1)
    assert f"{choice[0]},{choice[1]}" in timings and len(timings) == len(BT.CANDIDATES)
    choice2, timings2 = BT.autotune(rm, rm, cache=cache)
    assert choice2 == choice and timings2 == timings
