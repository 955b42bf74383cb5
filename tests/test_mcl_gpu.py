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


MCL_RECOVERY = ((1e-2, 30, 40, 0.9), (5e-3, 20, 30, 0.95), (2e-2, 10, 25, 0.8), (3e-2, 5, 12, 0.9))


class _Sizing:
    """Learned sizing needs a model on the context: one trained on A*A's
    exact counts, dropped afterwards."""

    def __init__(self, sizing_mode, A):
        self.m = None
        if sizing_mode == "learned":
            from combblas_gb300 import sizing

            feat, _, nnz = sizing.features(A, A)
            self.m = sizing.SizingModel(seed=0)
            self.m.fit(feat, nnz, steps=300)

    def __enter__(self):
        if self.m is not None:
            self.m.use()
        return self

    def __exit__(self, *exc):
        if self.m is not None:
            self.m.close()


@pytest.mark.parametrize("sizing", ["exact", "learned"])
def test_mcl_recovery_golden(gpu_ctx, oracle_lib, golden, sizing):
    """recoverNum > 0 (ParFriends.h:290-330), bit-exact against the
    reference's own MemEfficientSpGEMM output."""
    O = oracle_lib
    M = golden_matrix(golden, "mcl4096")
    with _Sizing(sizing, M):
        results = [mcl.mcl_expand(M, thr, k, sizing=sizing, recoverNum=rn, recoverPct=pct)[0]
                   for thr, k, rn, pct in MCL_RECOVERY]
    for (thr, k, rn, pct), R in zip(MCL_RECOVERY, results):
        cp, rows, vals = O.canonical_csc(*R.to_csc())
        key = f"mclrec/mcl4096/{thr:g}/{k}/{rn}/{pct:g}"
        gcp, grows, gvals = O.tuples_to_csc(golden[f"{key}/rows"], golden[f"{key}/cols"], golden[f"{key}/vals"],
                                            M.ncol)
        assert np.array_equal(cp, gcp) and np.array_equal(rows, grows) and np.array_equal(vals, gvals), (thr, k)


def test_mcl_recovery_vs_oracle_planted(gpu_ctx, oracle_lib):
    """The application's defaults (select 1100, recover 1400, 0.9) and a
    recovery-heavy setting on a planted graph, against the restatement."""
    O = oracle_lib
    M = G.mcl_planted(1 << 14, 256, 24, 6, seed=3)
    pcp, prow, pval = O.port_spgemm(M, M, O.SR_PLUSTIMES_F32, sorted=False)
    for thr, k, rn, pct in ((1e-4, 1100, 1400, 0.9), (2e-3, 40, 80, 0.95)):
        R, _ = mcl.mcl_expand(M, thr, k, recoverNum=rn, recoverPct=pct)
        cp, rows, vals = O.canonical_csc(*R.to_csc())
        ecp, erow, evals = O.canonical_csc(*O.port_mcl_select(pcp, prow, pval, thr, k, rn, pct))
        assert np.array_equal(cp, ecp) and np.array_equal(rows, erow) and np.array_equal(vals, evals), (thr, k)


def _device(M):
    """M as a device result (identity * M on the GPU keeps it exactly)."""
    n = M.nrow
    I = G.CSC(n, n, np.arange(n + 1), np.arange(n), np.ones(n, np.float32))
    return local.spgemm(I, M, dtype=np.float32)


def test_mcl_vector_steps(gpu_ctx, oracle_lib, golden):
    """MakeColStochastic / Inflate / Chaos on the device: bit-exact against
    the restatement, within 1e-6 of the reference's own steps."""
    O = oracle_lib
    M = golden_matrix(golden, "mcl4096")
    M.values = np.asarray(M.values, np.float32)
    cp, v = np.asarray(M.colptr), M.values
    R = mcl.MakeColStochastic(_device(M))
    _, _, sc = R.to_csc()
    assert np.array_equal(sc, O.port_mcl_colscale(cp, v))
    assert np.max(np.abs(sc - golden["mclstep/mcl4096/colscale"]) / sc) < 1e-6
    for power in (2.0, 1.5):
        _, _, iv = mcl.Inflate(_device(M), power).to_csc()
        assert np.array_equal(iv, golden[f"mclstep/mcl4096/inflate/{power:g}"]), power
    c = mcl.Chaos(_device(M))
    assert c == O.port_mcl_chaos(cp, v)
    assert abs(c - float(golden["mclstep/mcl4096/chaos"][0])) <= 1e-6 * c


MCL_LOOPS = ((2.0, 1e-4, 30, 40, 0.9, 0), (1.5, 1e-3, 20, 30, 0.9, 0), (2.0, 1e-4, 30, 40, 0.9, 2))


@pytest.mark.parametrize("infl,thr,k,rn,pct,mi", MCL_LOOPS)
def test_mcl_loop_golden(gpu_ctx, oracle_lib, golden, infl, thr, k, rn, pct, mi):
    """The whole HipMCL loop in one call, the matrix on the device between
    iterations: bit-exact against the restated loop (same iteration count
    and chaos), and against the reference's own loop bit-exact once
    converged, within 1e-5 relative after two iterations."""
    O = oracle_lib
    M = golden_matrix(golden, "mcl4096")
    R, it, chaos = mcl.HipMCL(M, infl, thr, k, rn, pct, max_iter=mi)
    cp, rows, vals = O.canonical_csc(*R.to_csc())
    (pcp, prow, pval), pit, pchaos = O.port_mcl_iterate(M, infl, thr, k, rn, pct, mi)
    assert it == pit and np.float32(chaos) == np.float32(pchaos)
    assert np.array_equal(cp, pcp) and np.array_equal(rows, prow) and np.array_equal(vals, pval)
    key = f"mclloop/mcl4096/{infl:g}/{thr:g}/{k}/{rn}/{pct:g}/{mi}"
    assert it == int(golden[f"{key}/iterations"][0])
    assert np.array_equal(cp, golden[f"{key}/colptr"]) and np.array_equal(rows, golden[f"{key}/rowidx"])
    gv = golden[f"{key}/values"]
    if mi == 0:
        assert np.array_equal(vals, gv)
    else:
        assert np.max(np.abs(vals - gv) / gv) < 1e-5


@pytest.mark.parametrize("sizing", ["exact", "learned"])
def test_mcl_loop_planted_vs_oracle(gpu_ctx, oracle_lib, sizing):
    """A larger planted graph with the application's defaults, three
    iterations, against the restated loop."""
    O = oracle_lib
    M = G.mcl_planted(1 << 14, 256, 24, 6, seed=11)
    with _Sizing(sizing, M):
        R, it, chaos = mcl.HipMCL(M, 2.0, 1e-4, 1100, 1400, 0.9, sizing=sizing, max_iter=3)
    cp, rows, vals = O.canonical_csc(*R.to_csc())
    (pcp, prow, pval), pit, pchaos = O.port_mcl_iterate(M, 2.0, 1e-4, 1100, 1400, 0.9, 3)
    assert it == pit == 3 and np.float32(chaos) == np.float32(pchaos)
    assert np.array_equal(cp, pcp) and np.array_equal(rows, prow) and np.array_equal(vals, pval)
