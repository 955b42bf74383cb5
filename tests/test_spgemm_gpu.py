"""GPU SpGEMM through the C ABI against the reference's golden outputs and
the oracle's C restatement.

PlusTimes fp64 runs under both folds: "ordered" (the reference's hash-path
left fold, bit-exact against the reference's hash variants and the oracle)
and "exact" (the default: each entry the exact sum of the rounded products,
rounded once -- bit-exact against the oracle's exact fold, within 1e-12 of
the reference)."""
import numpy as np
import pytest

from combblas_gb300 import generators as G
from combblas_gb300 import local
from conftest import golden_matrix
from test_oracle import prod_cases, typed

pytestmark = pytest.mark.gpu

SR_NAME = {0: ("plustimes", np.float64), 1: ("plustimes", np.float32), 2: ("plustimes", np.int64),
           3: ("minplus", np.float64), 4: ("select2ndmin", np.int64), 5: ("bool", np.bool_),
           6: ("minplus", np.int64)}
TOL = {0: 1e-12, 1: 1e-5}  # PlusTimes fp64 / fp32 (relative), against the hybrid's heap columns


FOLDS = ["ordered", "exact"]


def gpu_csc(A, B, sr, fold="ordered", **kw):
    name, dt = SR_NAME[sr]
    R = local.spgemm(A, B, sr=name, dtype=dt, fold=fold, **kw)
    return R.to_csc()


def port(O, A, B, sr, fold="ordered", **kw):
    """The oracle's product under the fold the GPU ran with (the fold only
    changes PlusTimes fp64)."""
    return O.port_spgemm(A, B, sr, fold=fold if sr == 0 else "ordered", **kw)


def assert_same(cp, rows, vals, ecp, erows, evals, sr=None, exact=True, what=""):
    assert np.array_equal(cp, ecp), what
    assert np.array_equal(rows, erows), what
    if exact or sr not in TOL:
        assert np.array_equal(vals, evals), what
    else:
        rel = np.abs(vals - evals) / np.maximum(np.abs(evals), np.finfo(evals.dtype).tiny)
        assert rel.max(initial=0) <= TOL[sr], (what, rel.max())


@pytest.mark.parametrize("fold", FOLDS)
def test_golden_products(gpu_ctx, oracle_lib, golden, fold):
    O = oracle_lib
    g = golden
    for key in prod_cases(g):
        _, name, kind, _ = key.split("/")
        sr = int(g[f"{key}/sr"])
        variant = int(g[f"{key}/variant"])
        if name == "galerkin4":
            continue
        if name == "rand_dcsc":
            A = typed(golden_matrix(g, "rand_dcsc"), sr, 3, O)
            B = typed(golden_matrix(g, "rand_dcsc_B"), sr, 4, O)
        else:
            M = golden_matrix(g, name)
            A = typed(M, sr, 1, O)
            B = A if kind != "AAt" else typed(G.transpose(M), sr, 2, O)
        cp, rows, vals = gpu_csc(A, B, sr, fold)
        ecp, erows, evals = O.tuples_to_csc(g[f"{key}/rows"], g[f"{key}/cols"], g[f"{key}/vals"], B.ncol)
        exact = variant in (O.V_HASH_SORTED, O.V_HASH_UNSORTED) and (fold == "ordered" or sr != 0)
        assert_same(cp, rows, vals, ecp, erows, evals, sr, exact, key)
        # bit-exact against the oracle under the same fold
        pcp, prow, pval = port(O, A, B, sr, fold)
        assert_same(cp, rows, vals, pcp, prow, pval, sr, True, key + " vs port")


@pytest.mark.parametrize("fold", FOLDS)
def test_golden_galerkin(gpu_ctx, oracle_lib, golden, fold):
    """Galerkin values are small integers: every fold gives them exactly."""
    O = oracle_lib
    A = golden_matrix(golden, "poisson4")
    R = golden_matrix(golden, "agg4")
    Rt = G.transpose(R)
    cp, rows, vals = gpu_csc(A, Rt, 0, fold)
    AR = G.CSC(A.nrow, Rt.ncol, cp, rows, vals)
    cp2, rows2, vals2 = gpu_csc(R, AR, 0, fold)
    key = "prod/galerkin4/RAR/0"
    ecp, erows, evals = O.tuples_to_csc(golden[f"{key}/rows"], golden[f"{key}/cols"], golden[f"{key}/vals"], AR.ncol)
    assert_same(cp2, rows2, vals2, ecp, erows, evals, 0, True, key)


@pytest.mark.parametrize("fold", FOLDS)
@pytest.mark.parametrize("scale,ef", [(12, 8), (14, 8), (15, 4)])
def test_rmat_fp64_bitexact_vs_port(gpu_ctx, oracle_lib, scale, ef, fold):
    O = oracle_lib
    A = G.rmat(scale, ef, seed=scale)
    cp, rows, vals = gpu_csc(A, A, 0, fold)
    pcp, prow, pval = port(O, A, A, 0, fold)
    assert_same(cp, rows, vals, pcp, prow, pval, 0, True, f"rmat{scale}")
    # repeated runs are bit-identical
    cp2, rows2, vals2 = gpu_csc(A, A, 0, fold)
    assert np.array_equal(vals, vals2) and np.array_equal(rows, rows2)
    if fold == "exact":  # and within the reference's rounding of the hash-path fold
        ocp, orow, oval = O.port_spgemm(A, A, O.SR_PLUSTIMES_F64)
        assert_same(cp, rows, vals, ocp, orow, oval, 0, False, f"rmat{scale} exact vs ordered")


@pytest.mark.parametrize("opts", [{}, dict(tiny_limit=0, small_limit=0)])
def test_exact_fold_signed_zeros_and_fallback_columns(gpu_ctx, oracle_lib, opts):
    """Signed values, explicit +0.0/-0.0, exact cancellation, and columns
    whose products span too many binades (those keep the ordered fold):
    bit-exact against the oracle's exact fold, which applies the same
    column admission."""
    O = oracle_lib
    rng = np.random.default_rng(11)
    A = G.random_sparse(3000, 3000, 0.004, seed=12)
    e = np.where(rng.random(A.nnz) < 0.97, rng.integers(-12, 12, A.nnz), rng.integers(-300, 300, A.nnz))
    A.values = rng.standard_normal(A.nnz) * np.exp2(e.astype(np.float64))
    A.values[rng.random(A.nnz) < 0.03] = 0.0
    A.values[rng.random(A.nnz) < 0.03] = -0.0
    cp, rows, vals = gpu_csc(A, A, 0, "exact", **opts)
    pcp, prow, pval = port(O, A, A, 0, "exact")
    assert np.array_equal(cp, pcp) and np.array_equal(rows, prow)
    assert np.array_equal(vals.view(np.int64), pval.view(np.int64))  # signs of zero included


@pytest.mark.parametrize("sr", [1, 2, 3, 4, 5, 6])
def test_rmat_semirings_vs_port(gpu_ctx, oracle_lib, sr):
    O = oracle_lib
    A = typed(G.rmat(13, 6, seed=21), sr, 5, O)
    cp, rows, vals = gpu_csc(A, A, sr)
    pcp, prow, pval = O.port_spgemm(A, A, sr)
    assert_same(cp, rows, vals, pcp, prow, pval, sr, True, f"sr{sr}")


@pytest.mark.parametrize("opts", [dict(tile_rows=8192), dict(tile_rows=4096),
                                  dict(tile_rows=8192, tiny_limit=64, small_limit=1024),
                                  dict(tiny_limit=0, small_limit=0)])
@pytest.mark.parametrize("sr,fold", [(0, "ordered"), (0, "exact"), (5, "ordered")])
def test_tile_and_class_options_vs_port(gpu_ctx, oracle_lib, opts, sr, fold):
    """Row-tile height and warp-path limits change the schedule, never the
    result: every option set is bit-exact against the oracle."""
    O = oracle_lib
    A = typed(G.rmat(15, 8, seed=5), sr, 7, O)
    cp, rows, vals = gpu_csc(A, A, sr, fold, **opts)
    pcp, prow, pval = port(O, A, A, sr, fold)
    assert_same(cp, rows, vals, pcp, prow, pval, sr, True, str(opts))


@pytest.mark.parametrize("fold", FOLDS)
def test_tall_matrix_many_tiles(gpu_ctx, oracle_lib, fold):
    """m > 1M rows: several row tiles and several symbolic bitmaps (beyond
    the exact kernel's bucketing limit: its per-tile enumeration mode)."""
    O = oracle_lib
    A = G.random_sparse(1_500_000, 400, 2e-5, seed=2)
    B = G.random_sparse(400, 300, 0.05, seed=3)
    cp, rows, vals = gpu_csc(A, B, 0, fold, tiny_limit=0, small_limit=0)
    pcp, prow, pval = port(O, A, B, 0, fold)
    assert_same(cp, rows, vals, pcp, prow, pval, 0, True, "tall")


def test_dcsc_inputs_and_views(gpu_ctx, oracle_lib):
    O = oracle_lib
    A = G.random_sparse(500, 400, 0.01, seed=8, empty_cols=0.4)
    B = G.random_sparse(400, 350, 0.02, seed=9, empty_cols=0.4)
    Ad, Bd = local.DCSC.from_csc(A), local.DCSC.from_csc(B)
    R = local.spgemm(Ad, Bd, keep_empty=True)
    cp, jc, ir, num = R.to_host()
    assert np.array_equal(jc, Bd.jc)  # SpTuples view: one column per stored column of B
    full, rows, vals = R.to_csc()
    pcp, prow, pval = port(O, A, B, 0, "exact")  # the default fold
    assert_same(full, rows, vals, pcp, prow, pval, 0, True, "dcsc")
    R2 = local.spgemm(Ad, Bd, keep_empty=False)  # SpDCCols view drops empty output columns
    cp2, jc2, ir2, num2 = R2.to_host()
    nzcols = np.nonzero(np.diff(pcp))[0]
    assert np.array_equal(jc2, nzcols) and np.array_equal(ir2, prow) and np.array_equal(num2, pval)


def test_device_resident_inputs(gpu_ctx, oracle_lib):
    O = oracle_lib
    A = G.rmat(11, 8, seed=4)
    Ad = local.DeviceMatrix.from_host(A)
    cp, rows, vals = local.spgemm(Ad, Ad).to_csc()
    pcp, prow, pval = port(O, A, A, 0, "exact")
    assert_same(cp, rows, vals, pcp, prow, pval, 0, True, "device")


def test_edge_cases(gpu_ctx, oracle_lib):
    O = oracle_lib
    # empty operands -> empty product with the right shape (mtSpGEMM.h:224-227)
    Z = G.CSC(50, 40, np.zeros(41, np.int64), np.zeros(0, np.int64), np.zeros(0))
    B = G.random_sparse(40, 30, 0.1, seed=1)
    R = local.spgemm(Z, B)
    assert R.nnz == 0 and R.nrow == 50 and R.ncol == 30
    # 1x1
    one = G.CSC(1, 1, np.array([0, 1]), np.array([0]), np.array([3.0]))
    cp, rows, vals = local.spgemm(one, one).to_csc()
    assert list(rows) == [0] and list(vals) == [9.0]
    # a fully dense column in A and in B
    A = G.random_sparse(300, 300, 0.01, seed=2)
    dense_rows = np.arange(300)
    rows = np.concatenate([A.rowidx, dense_rows])
    cols = np.concatenate([A.col_ids(), np.full(300, 7)])
    D = G.csc_from_coo(300, 300, rows, cols)
    D.values = np.linspace(0.1, 1.0, D.nnz)
    for fold in FOLDS:
        cp, rows, vals = local.spgemm(D, D, fold=fold).to_csc()
        pcp, prow, pval = port(O, D, D, 0, fold)
        assert_same(cp, rows, vals, pcp, prow, pval, 0, True, "dense column " + fold)


def test_errors_are_reported(gpu_ctx):
    from combblas_gb300._lib import GbcError

    A = G.random_sparse(30, 20, 0.2, seed=1)
    with pytest.raises(GbcError, match="inner dimensions"):
        local.spgemm(A, A)
    # rows not ascending within a column: rejected by the validation pass
    bad = G.CSC(4, 2, np.array([0, 2, 3]), np.array([3, 1, 0]), np.ones(3))
    sq = G.CSC(2, 2, np.array([0, 1, 2]), np.array([0, 1]), np.ones(2))
    with pytest.raises(GbcError, match="ascending"):
        local.spgemm(bad, sq)
    # row id out of range
    bad2 = G.CSC(4, 2, np.array([0, 1, 2]), np.array([1, 9]), np.ones(2))
    with pytest.raises(GbcError, match="out of range"):
        local.spgemm(bad2, sq)


def test_colstats_vs_reference(gpu_ctx, golden):
    for name in ("seven", "nonsym", "torus", "bcsstk01", "rmat8"):
        M = golden_matrix(golden, name)
        D = local.DCSC.from_csc(M)
        flop = local.estimateFLOP(D, D)
        nnz = local.estimateNNZ_Hash(D, D)
        assert np.array_equal(flop, golden[f"colstats/{name}/flop"]), name
        assert np.array_equal(nnz, golden[f"colstats/{name}/nnz"]), name


def content_hash(cp, rows, vals, cols=None):
    """Host restatement of the phased checksum: wrap-around sum over entries
    of mix64(((col << 32) ^ row) * 0x9e3779b97f4a7c15 ^ value bits)."""
    u = np.uint64
    ncol = len(cp) - 1
    col = np.repeat(np.arange(ncol, dtype=np.uint64) if cols is None else np.asarray(cols, np.uint64),
                    np.diff(cp))
    bits = np.asarray(vals).view(np.uint64 if np.asarray(vals).dtype.itemsize == 8 else np.uint32).astype(u)
    with np.errstate(over="ignore"):
        x = ((col << u(32)) ^ rows.astype(u)) * u(0x9E3779B97F4A7C15) ^ bits
        x ^= x >> u(31)
        x *= u(0x7FB5D329728EA185)
        x ^= x >> u(27)
        x *= u(0x81DADEF4BC2DD44D)
        x ^= x >> u(33)
        return int(np.sum(x, dtype=u))


@pytest.mark.parametrize("fold", FOLDS)
def test_phased_matches_single_pass(gpu_ctx, oracle_lib, fold):
    """Column phases (small budget -> many phases) give the same nnz and
    checksums as the single-pass product and the oracle."""
    O = oracle_lib
    A = G.rmat(13, 8, seed=6)
    cp, rows, vals = gpu_csc(A, A, 0, fold)
    pcp, prow, pval = port(O, A, A, 0, fold)
    ref_rows = int(prow.sum())
    ref_hash = content_hash(pcp, prow, pval)
    assert content_hash(cp, rows, vals) == ref_hash
    for budget in (len(rows), 200_000, 50_000):
        st = local.spgemm_phased(A, A, max_phase_nnz=budget, fold=fold)
        assert st.nnz == len(prow) and st.row_checksum == ref_rows
        assert st.content_hash == ref_hash
        assert abs(st.val_checksum - pval.sum()) <= 1e-9 * abs(pval.sum())
        assert st.phases >= (len(prow) + budget - 1) // budget
        assert st.alloc_nnz == st.nnz and st.overflow_cols == 0
        assert st.flops == int(O.port_spgemm(A, A, O.SR_PLUSTIMES_F64, want_counts=True)[1][0].sum())


@pytest.mark.parametrize("margin,fold", [(None, "exact"), (0.0, "exact"), (0.0, "ordered")])
def test_phased_learned_identical_to_exact(gpu_ctx, oracle_lib, margin, fold):
    """Learned phase sizing (model trained on another seed of the same
    class; margin 0 forces many overflow re-runs) gives the exact product's
    nnz, row checksum and content hash."""
    from combblas_gb300 import sizing
    O = oracle_lib
    A = G.rmat(14, 8, seed=43)
    Atrain = G.rmat(14, 8, seed=44)
    feat, flop, nnz = sizing.features(Atrain, Atrain)
    m = sizing.SizingModel(seed=1)
    m.fit(feat, nnz, steps=300)
    if margin is not None:
        m.set_margin(margin)
    m.use()
    try:
        pcp, prow, pval = port(O, A, A, 0, fold)
        ref_hash = content_hash(pcp, prow, pval)
        for budget in (1 << 40, 400_000):
            ex = local.spgemm_phased(A, A, max_phase_nnz=budget, fold=fold)
            le = local.spgemm_phased(A, A, max_phase_nnz=budget, sizing="learned", fold=fold)
            assert ex.content_hash == ref_hash
            assert (le.nnz, le.row_checksum, le.content_hash) == (ex.nnz, ex.row_checksum, ex.content_hash)
            assert le.alloc_nnz >= 1 and le.flops == ex.flops
            if margin == 0.0:
                assert le.overflow_cols > 0
    finally:
        m.close()


def test_exact_kernel_visits_both_tile_paths(gpu_ctx, oracle_lib):
    """The exact-fold kernel's two tile paths -- dense accumulator visits and
    sorted ranges of light tiles -- both run on an R-MAT product with
    4096-row tiles, and the product is bit-exact against the oracle's exact
    fold (the two paths' thresholds change which tiles take which path, not
    the values: the bench records identical content hashes across them)."""
    O = oracle_lib
    A = G.rmat(16, 16, seed=21)
    cols = np.sort(np.random.default_rng(3).choice(A.ncol, 3000, replace=False))
    cnt = np.diff(A.colptr)[cols]
    cp = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    idx = np.concatenate([np.arange(A.colptr[c], A.colptr[c + 1]) for c in cols])
    B = G.CSC(A.nrow, len(cols), cp, A.rowidx[idx], A.values[idx])
    R = local.spgemm(A, B, fold="exact", tile_rows=4096)
    st = R.stats
    assert st.tile_visits_dense > 0 and st.tile_visits_range > 0, (st.tile_visits_dense, st.tile_visits_range)
    got = R.to_csc()
    exp = O.port_spgemm(A, B, O.SR_PLUSTIMES_F64, fold="exact")
    assert all(np.array_equal(np.asarray(x).view(np.int64) if np.asarray(x).dtype == np.float64 else x,
                              np.asarray(y).view(np.int64) if np.asarray(y).dtype == np.float64 else y)
               for x, y in zip(got, exp))
