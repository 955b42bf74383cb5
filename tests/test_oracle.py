"""The oracle against the reference's own outputs (golden fixtures made by
running the reference) -- CPU only."""
import numpy as np
import pytest

from combblas_gb300 import generators as G
from conftest import golden_matrix

SR_TOL = {0: 1e-12, 1: 1e-5}  # PlusTimes fp64 / fp32 relative tolerance vs the hybrid's heap columns


def typed(M, sr, seed, O):
    dt = O.SR_DTYPE[sr]
    rng = np.random.default_rng(seed)
    if dt == np.bool_:
        return M.with_values(np.ones(M.nnz, np.bool_))
    if dt == np.int64:
        return M.with_values(rng.integers(1, 50, M.nnz).astype(np.int64))
    if M.values is None:
        return M.with_values((1.0 - rng.random(M.nnz)).astype(dt))
    return M.astype(dt)


def prod_cases(g):
    keys = sorted({k.rsplit("/", 1)[0] for k in g.files if k.startswith("prod/") and k.endswith("/rows")})
    return keys


def check_csc(cp, rows, vals, g, key, sr, variant, ncol, O, exact_values):
    gcp, grows, gvals = O.tuples_to_csc(g[f"{key}/rows"], g[f"{key}/cols"], g[f"{key}/vals"], ncol)
    if variant == O.V_HASH_UNSORTED:
        cp, rows, vals = O.canonical_csc(cp, rows, vals)
    assert np.array_equal(cp, gcp), key
    assert np.array_equal(rows, grows), key
    if exact_values or sr not in SR_TOL:
        assert np.array_equal(vals, gvals), key
    else:
        rel = np.abs(vals - gvals) / np.maximum(np.abs(gvals), np.finfo(gvals.dtype).tiny)
        assert rel.max(initial=0) <= SR_TOL[sr], (key, rel.max())


def test_port_matches_reference_products(oracle_lib, golden):
    O = oracle_lib
    g = golden
    for key in prod_cases(g):
        _, name, kind, sr = key.split("/")
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
        sorted_ = variant != O.V_HASH_UNSORTED
        cp, rows, vals = O.port_spgemm(A, B, sr, sorted=sorted_)
        # the port follows the hash path's summation order: bit-exact against
        # the hash variants, within tolerance of the hybrid/heap ones
        exact = variant in (O.V_HASH_SORTED, O.V_HASH_UNSORTED)
        check_csc(cp, rows, vals, g, key, sr, variant, B.ncol, O, exact)
        if variant == O.V_HASH_UNSORTED:
            # slot order of the unsorted hash gather is reproduced exactly
            _, prow, pval = O.port_spgemm(A, B, sr, sorted=False)
            assert np.array_equal(prow, g[f"{key}/rows"]) and np.array_equal(pval, g[f"{key}/vals"])


def test_port_galerkin(oracle_lib, golden):
    O = oracle_lib
    g = golden
    A = golden_matrix(g, "poisson4")
    R = golden_matrix(g, "agg4")
    Rt = G.transpose(R)
    cp, rows, vals = O.port_spgemm(A, Rt, O.SR_PLUSTIMES_F64)
    AR = G.CSC(A.nrow, Rt.ncol, cp, rows, vals)
    cp2, rows2, vals2 = O.port_spgemm(R, AR, O.SR_PLUSTIMES_F64)
    key = "prod/galerkin4/RAR/0"
    check_csc(cp2, rows2, vals2, g, key, 0, 0, AR.ncol, O, exact_values=True)


def test_port_colstats(oracle_lib, golden):
    O = oracle_lib
    for name in ("seven", "nonsym", "torus", "bcsstk01", "rmat8"):
        M = golden_matrix(golden, name)
        (_, _, _), (flop, nnz) = O.port_spgemm(M, M, O.SR_PLUSTIMES_F64, want_counts=True)
        nz = np.diff(M.colptr) > 0
        assert np.array_equal(flop[nz], golden[f"colstats/{name}/flop"])
        assert np.array_equal(nnz[nz], golden[f"colstats/{name}/nnz"])


def test_port_bfs(oracle_lib, golden):
    O = oracle_lib
    for name in ("seven_sym", "torus", "rmat8"):
        M = golden_matrix(golden, name).with_values(None)
        for s in golden[f"bfs/{name}/sources"]:
            par, lev, it = O.port_bfs(M, int(s))
            assert np.array_equal(par, golden[f"bfs/{name}/{s}/parents"]), (name, s)
            assert np.array_equal(lev, golden[f"bfs/{name}/{s}/levels"]), (name, s)
            assert it == int(golden[f"bfs/{name}/{s}/iters"])


def test_port_spmspv(oracle_lib, golden):
    O = oracle_lib
    M = golden_matrix(golden, "rmat8").with_values(None)
    yr, yv = O.port_spmspv(M, golden["spmspv/rmat8/x_ind"], golden["spmspv/rmat8/x_val"])
    assert np.array_equal(yr, golden["spmspv/rmat8/y_ind"])
    assert np.array_equal(yv, golden["spmspv/rmat8/y_val"])


def test_port_mcl(oracle_lib, golden):
    O = oracle_lib
    M = golden_matrix(golden, "mcl4096")
    for thr, k in ((1e-4, 30), (1e-3, 12)):
        cp, rows, vals = O.port_spgemm(M, M, O.SR_PLUSTIMES_F32, sorted=False)
        scp, srows, svals = O.port_mcl_select(cp, rows, vals, thr, k)
        scp, srows, svals = O.canonical_csc(scp, srows, svals)
        key = f"mcl/mcl4096/{thr:g}/{k}"
        gcp, grows, gvals = O.tuples_to_csc(golden[f"{key}/rows"], golden[f"{key}/cols"], golden[f"{key}/vals"],
                                            M.ncol)
        assert np.array_equal(scp, gcp) and np.array_equal(srows, grows) and np.array_equal(svals, gvals)


def test_port_spmspv_semirings(oracle_lib, golden):
    """Select2nd (boolean optbuf path), SelectMax and PlusTimes SpMXSpV
    restated, against the reference's own output on a rectangular matrix."""
    O = oracle_lib
    R = golden_matrix(golden, "rect1500")
    x = golden["spmspvsr/x_ind"]
    for sx in (O.SX_SELECT2ND, O.SX_SELECTMAX):
        r, v = O.port_spmspv_sr(R, sx, x, golden["spmspvsr/x_i64"])
        assert np.array_equal(r, golden[f"spmspvsr/{sx}/y_ind"]) and np.array_equal(v, golden[f"spmspvsr/{sx}/y_val"])
    for dt in (np.float64, np.float32):
        name = np.dtype(dt).name
        r, v = O.port_spmspv_sr(R.with_values(R.values.astype(dt)), O.SX_PLUSTIMES, x,
                                golden["spmspvsr/x_f64"].astype(dt), dt)
        assert np.array_equal(r, golden[f"spmspvsr/3/{name}/y_ind"])
        assert np.array_equal(v, golden[f"spmspvsr/3/{name}/y_val"])
    Ri = R.with_values(np.round(R.values * 100).astype(np.int64))
    r, v = O.port_spmspv_sr(Ri, O.SX_PLUSTIMES, x, golden["spmspvsr/x_i64"], np.int64)
    assert np.array_equal(r, golden["spmspvsr/3/int64/y_ind"]) and np.array_equal(v, golden["spmspvsr/3/int64/y_val"])


MCL_RECOVERY = ((1e-2, 30, 40, 0.9), (5e-3, 20, 30, 0.95), (2e-2, 10, 25, 0.8), (3e-2, 5, 12, 0.9))


@pytest.mark.parametrize("thr,k,rn,pct", MCL_RECOVERY)
def test_port_mcl_recovery(oracle_lib, golden, thr, k, rn, pct):
    """MCLPruneRecoverySelect with recoverNum > 0 (ParFriends.h:290-330)
    against the reference's own MemEfficientSpGEMM output."""
    O = oracle_lib
    M = golden_matrix(golden, "mcl4096")
    cp, rows, vals = O.port_spgemm(M, M, O.SR_PLUSTIMES_F32, sorted=False)
    scp, srows, svals = O.canonical_csc(*O.port_mcl_select(cp, rows, vals, thr, k, rn, pct))
    key = f"mclrec/mcl4096/{thr:g}/{k}/{rn}/{pct:g}"
    gcp, grows, gvals = O.tuples_to_csc(golden[f"{key}/rows"], golden[f"{key}/cols"], golden[f"{key}/vals"], M.ncol)
    assert np.array_equal(scp, gcp) and np.array_equal(srows, grows) and np.array_equal(svals, gvals)
    # recovery changed the outcome: more entries than the same step without it
    ncp, _, _ = O.port_mcl_select(cp, rows, vals, thr, k)
    assert gcp[-1] > ncp[-1]


def test_port_mcl_vector_steps(oracle_lib, golden):
    """MakeColStochastic / Inflate / Chaos (MCL.cpp:389-449).  The port's
    column sums are exact sums rounded once, the reference's a left fold in
    storage order: scaled values agree within 1e-6 relative (fp32 tolerance
    1e-5); Inflate is bit-exact; Chaos agrees within 1e-6."""
    O = oracle_lib
    M = golden_matrix(golden, "mcl4096")
    cp, v = np.asarray(M.colptr), np.asarray(M.values, np.float32)
    sc = O.port_mcl_colscale(cp, v)
    ref = golden["mclstep/mcl4096/colscale"]
    assert np.max(np.abs(sc - ref) / ref) < 1e-6
    for power in (2.0, 1.5):
        assert np.array_equal(O.port_mcl_inflate(v, power), golden[f"mclstep/mcl4096/inflate/{power:g}"])
    c = O.port_mcl_chaos(cp, v)
    assert abs(c - float(golden["mclstep/mcl4096/chaos"][0])) <= 1e-6 * abs(c)
    # stochastic columns sum to 1 within rounding; a zero column stays zero
    sums = np.add.reduceat(sc.astype(np.float64), cp[:-1][np.diff(cp) > 0])
    assert np.all(np.abs(sums - 1.0) < 1e-5)


MCL_LOOPS = ((2.0, 1e-4, 30, 40, 0.9, 0), (1.5, 1e-3, 20, 30, 0.9, 0), (2.0, 1e-4, 30, 40, 0.9, 2))


@pytest.mark.parametrize("infl,thr,k,rn,pct,mi", MCL_LOOPS)
def test_port_mcl_loop(oracle_lib, golden, infl, thr, k, rn, pct, mi):
    """The HipMCL loop (MCL.cpp:526-626) restated against the reference's
    own loop: converged runs end bit-identical after the same number of
    iterations; a two-iteration run has the same pattern and values within
    the fp32 tolerance (1e-5 relative)."""
    O = oracle_lib
    M = golden_matrix(golden, "mcl4096")
    (cp, rows, vals), it, chaos = O.port_mcl_iterate(M, infl, thr, k, rn, pct, mi)
    key = f"mclloop/mcl4096/{infl:g}/{thr:g}/{k}/{rn}/{pct:g}/{mi}"
    assert it == int(golden[f"{key}/iterations"][0])
    assert np.array_equal(cp, golden[f"{key}/colptr"]) and np.array_equal(rows, golden[f"{key}/rowidx"])
    gv = golden[f"{key}/values"]
    if mi == 0:
        assert np.array_equal(vals, gv) and chaos <= 0.0001
    else:
        assert np.max(np.abs(vals - gv) / gv) < 1e-5
        assert abs(chaos - float(golden[f"{key}/chaos"][0])) <= 1e-5 * chaos


def test_reference_build_reproduces_golden(oracle_lib, golden):
    """Where the reference was compiled (this container), it still produces
    the committed fixtures."""
    O = oracle_lib
    if not O.have_ref():
        pytest.skip("reference sources not present")
    M = golden_matrix(golden, "rmat8")
    A = typed(M, O.SR_PLUSTIMES_F64, 1, O)
    r, c, v, _ = O.ref_spgemm(A, A, O.SR_PLUSTIMES_F64)
    key = "prod/rmat8/AA/0"
    assert np.array_equal(r, golden[f"{key}/rows"]) and np.array_equal(v, golden[f"{key}/vals"])


def test_oracle_detects_planted_error(oracle_lib, golden):
    """A mistake planted in the oracle's output (on the CPU) is caught by the
    comparison used throughout the tests."""
    O = oracle_lib
    M = golden_matrix(golden, "rmat8")
    A = typed(M, O.SR_PLUSTIMES_F64, 1, O)
    cp, rows, vals = O.port_spgemm(A, A, O.SR_PLUSTIMES_F64, sorted=True)
    vals = vals.copy()
    vals[len(vals) // 2] *= 1.0 + 1e-9
    with pytest.raises(AssertionError):
        check_csc(cp, rows, vals, golden, "prod/rmat8/AA_hash_sorted/0", 0, O.V_HASH_SORTED, A.ncol, O, True)


def test_port_msbfs(oracle_lib, golden):
    """The multi-source BFS loop over the C restatement reproduces the
    reference's own PSpGEMM<Select2ndMin> loop (golden), and away from the
    roots its parents are the single-source BFS parents."""
    O = oracle_lib
    for name in ("rmat8", "torus"):
        M = golden_matrix(golden, name).with_values(None)
        roots = golden[f"msbfs/{name}/roots"]
        par, lv = O.port_msbfs(M, roots)
        assert np.array_equal(par, golden[f"msbfs/{name}/parents"]), name
        assert lv == int(golden[f"msbfs/{name}/levels"])
        for r, s in enumerate(roots):
            single, _, _ = O.port_bfs(M, int(s))
            other = np.arange(M.ncol) != s
            assert np.array_equal(par[r][other], single[other]), (name, s)
            assert par[r][s] == s


def merge_lists(golden, K, sr, O):
    lists = [golden_matrix(golden, f"merge{k}") for k in range(K)]
    if sr != O.SR_PLUSTIMES_F64:
        lists = [typed(M, sr, 40 + k, O) for k, M in enumerate(lists)]
    return lists


def test_port_multiway_merge(oracle_lib, golden):
    """MultiwayMerge restated: exact against the reference for two lists and
    for min-type semirings; with more lists the reference's heap decides the
    order of equal keys, so fp64 sums agree within 1e-12."""
    O = oracle_lib
    for K in (2, 4):
        for sr in (O.SR_PLUSTIMES_F64, O.SR_SELECT2NDMIN_I64):
            lists = merge_lists(golden, K, sr, O)
            cp, rows, vals = O.port_multiway_merge(lists, 400, 250, sr)
            key = f"merge/{K}/{sr}"
            check_csc(cp, rows, vals, golden, key, sr, O.V_HYBRID, 250, O,
                      exact_values=(K == 2 or sr != O.SR_PLUSTIMES_F64))


def test_port_spmv(oracle_lib, golden):
    """dcsc_gespmv restated (column order, SR::axpy per entry) reproduces the
    reference's own multiply bit for bit."""
    O = oracle_lib
    M = golden_matrix(golden, "rmat8")
    for sr in (O.SR_PLUSTIMES_F64, O.SR_MINPLUS_F64, O.SR_SELECT2NDMIN_I64, O.SR_BOOL):
        y = O.port_spmv(typed(M, sr, 50 + sr, O), golden[f"spmv/{sr}/x"], golden[f"spmv/{sr}/y0"], sr)
        assert np.array_equal(y, golden[f"spmv/{sr}/y"]), sr


def _fsum_product(A, B):
    """Each entry of A*B as math.fsum of its products fl(a*b): the correctly
    rounded sum (an independent restatement of the exact fold)."""
    import math

    cps, rows, vals, negz = [0], [], [], []
    for j in range(B.ncol):
        ks = B.rowidx[B.colptr[j]:B.colptr[j + 1]]
        bv = B.values[B.colptr[j]:B.colptr[j + 1]]
        if len(ks) == 0:
            cps.append(cps[-1])
            continue
        rr = np.concatenate([A.rowidx[A.colptr[k]:A.colptr[k + 1]] for k in ks])
        pv = np.concatenate([A.values[A.colptr[k]:A.colptr[k + 1]] * b for k, b in zip(ks, bv)])
        order = np.argsort(rr, kind="stable")
        rr, pv = rr[order], pv[order]
        u, st = np.unique(rr, return_index=True)
        en = np.append(st[1:], len(rr))
        rows.append(u)
        vals.append(np.array([math.fsum(pv[s:e]) for s, e in zip(st, en)]))
        # fsum returns +0.0 for sums of -0.0 only; the fold keeps -0.0 there
        negz.append(np.array([bool(np.all((pv[s:e] == 0) & np.signbit(pv[s:e]))) for s, e in zip(st, en)]))
        cps.append(cps[-1] + len(u))
    v = np.concatenate(vals)
    v[np.concatenate(negz)] = -0.0
    return np.array(cps), np.concatenate(rows), v


@pytest.mark.parametrize("case", ["rmat", "signed"])
def test_port_exact_fold_is_fsum(oracle_lib, case):
    """The oracle's exact fold gives every entry as the correctly rounded
    sum of its rounded products (math.fsum), signs of zero included, on
    admitted columns; it stays within 1e-12 of the hash-path fold."""
    O = oracle_lib
    if case == "rmat":
        A = G.rmat(10, 8, seed=10)
    else:
        rng = np.random.default_rng(1)
        A = G.random_sparse(300, 300, 0.05, seed=3)
        A.values = rng.standard_normal(A.nnz) * np.exp2(rng.integers(-10, 10, A.nnz).astype(np.float64))
        A.values[rng.random(A.nnz) < 0.05] = 0.0
        A.values[rng.random(A.nnz) < 0.02] = -0.0
    cp, rows, vals = O.port_spgemm(A, A, O.SR_PLUSTIMES_F64, fold="exact")
    ecp, erows, evals = _fsum_product(A, A)
    assert np.array_equal(cp, ecp) and np.array_equal(rows, erows)
    assert np.array_equal(vals.view(np.int64), evals.view(np.int64))
    if case == "rmat":
        ocp, orow, oval = O.port_spgemm(A, A, O.SR_PLUSTIMES_F64)
        assert np.array_equal(orow, rows)
        assert np.max(np.abs(oval - vals) / np.abs(vals)) <= 1e-12
        assert np.mean(oval != vals) > 0.01  # the folds do differ in the last bits


def test_port_exact_fold_admission(oracle_lib):
    """A column whose product window spans more than 61 binades keeps the
    hash-path fold under fold="exact"; the other columns are exact."""
    O = oracle_lib
    rng = np.random.default_rng(2)
    A = G.random_sparse(200, 200, 0.08, seed=4)
    A.values = 1.0 + rng.random(A.nnz)
    wide = A.colptr[3], A.colptr[4]
    A.values[wide[0]] = 2.0 ** -80  # products with column 3 reach 80 binades below the rest
    x = O.port_spgemm(A, A, O.SR_PLUSTIMES_F64, fold="exact")
    o = O.port_spgemm(A, A, O.SR_PLUSTIMES_F64)
    f = _fsum_product(A, A)
    assert np.array_equal(x[0], o[0]) and np.array_equal(x[1], o[1])
    # columns j with B(3, j) != 0 (they use A's column 3) and column 3 itself
    # (its B values hold the small one) take the ordered fold, the rest are exact
    Bcols = set(np.nonzero([3 in A.rowidx[A.colptr[j]:A.colptr[j + 1]] for j in range(A.ncol)])[0].tolist()) | {3}
    for j in range(A.ncol):
        s, e = x[0][j], x[0][j + 1]
        want = o[2][s:e] if j in Bcols else f[2][s:e]
        assert np.array_equal(x[2][s:e], want), j
    assert len(Bcols) > 0 and any(not np.array_equal(o[2][x[0][j]:x[0][j + 1]], f[2][x[0][j]:x[0][j + 1]])
                                  for j in range(A.ncol) if j not in Bcols)
