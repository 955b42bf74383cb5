"""Regenerate tests/golden/golden.npz by running the reference itself.

Every expected output in the fixture file is produced by the reference's own
header templates (oracle/_ref/libcombblas_ref.so, compiled from the reference
sources by oracle/Makefile); inputs are the reference's in-repo matrix
fixtures (ReleaseTests/*.mtx, Applications/**/*.mtx) and seeded synthetic
matrices from combblas_gb300.generators.  Run here, where the reference is
present:

    python tests/golden/make_golden.py /root/reference

The GPU machine only reads the resulting .npz.
"""
from __future__ import annotations

import os
import sys

# The reference's BFS (PreAllocatedSPA with 4 buckets per thread) divides by
# zero on graphs smaller than its bucket count when several OpenMP threads
# run; results do not depend on the thread count, so fixtures use one.
os.environ["OMP_NUM_THREADS"] = "1"

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from combblas_gb300 import generators as G  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")


def read_mtx(path: str) -> G.CSC:
    with open(path) as f:
        lines = f.read().splitlines()
    header = lines[0] if lines and lines[0].startswith("%%") else ""
    symmetric = "symmetric" in header
    body = [l for l in lines if l.strip() and not l.startswith("%")]
    if header:
        m, n, nz = (int(x) for x in body[0].split()[:3])
        body = body[1:1 + nz]
    else:  # bare 1-based edge list (Applications/torus.mtx)
        idx = np.array([[int(x) for x in l.split()[:2]] for l in body])
        m = n = int(idx.max())
    rows, cols, vals = [], [], []
    for l in body:
        p = l.split()
        r, c = int(p[0]) - 1, int(p[1]) - 1
        v = float(p[2]) if len(p) > 2 else 1.0
        rows.append(r)
        cols.append(c)
        vals.append(v)
        if symmetric and r != c:
            rows.append(c)
            cols.append(r)
            vals.append(v)
    rows, cols, vals = np.array(rows), np.array(cols), np.array(vals)
    key = cols * m + rows
    order = np.argsort(key, kind="stable")
    return G.csc_from_coo(m, n, rows[order], cols[order], vals[order])


def put_mat(d, name, M):
    d[f"{name}/shape"] = np.array([M.nrow, M.ncol], np.int64)
    d[f"{name}/colptr"] = M.colptr
    d[f"{name}/rowidx"] = M.rowidx
    if M.values is not None:
        d[f"{name}/values"] = M.values


def put_prod(d, name, A, B, sr, variant=O.V_HYBRID):
    r, c, v, _ = O.ref_spgemm(A, B, sr, variant)
    d[f"{name}/sr"] = np.array(sr)
    d[f"{name}/variant"] = np.array(variant)
    d[f"{name}/rows"] = r
    d[f"{name}/cols"] = c
    d[f"{name}/vals"] = v


def with_type(M, sr, seed):
    dt = O.SR_DTYPE[sr]
    rng = np.random.default_rng(seed)
    if dt == np.bool_:
        return M.with_values(np.ones(M.nnz, np.bool_))
    if dt == np.int64:
        return M.with_values(rng.integers(1, 50, M.nnz).astype(np.int64))
    if M.values is None:
        return M.with_values((1.0 - rng.random(M.nnz)).astype(dt))
    return M.astype(dt)


def main(ref_root: str):
    if not O.have_ref():
        O.build(ref_root)
    d: dict = {}
    seven = read_mtx(os.path.join(ref_root, "ReleaseTests", "sevenvertex.mtx"))
    nonsym = read_mtx(os.path.join(ref_root, "ReleaseTests", "small_nonsym.mtx"))
    torus = read_mtx(os.path.join(ref_root, "Applications", "torus.mtx"))
    bcs = read_mtx(os.path.join(ref_root, "Applications", "Ordering", "bcsstk01.mtx"))
    rm = G.rmat(8, 8, seed=11)
    rm_dcsc = G.random_sparse(300, 260, 0.02, seed=5, empty_cols=0.3)
    inputs = {"seven": seven, "nonsym": nonsym, "torus": torus, "bcsstk01": bcs, "rmat8": rm, "rand_dcsc": rm_dcsc}
    for k, M in inputs.items():
        put_mat(d, f"in/{k}", M)
    cases = []
    for name in ("seven", "nonsym", "torus", "bcsstk01", "rmat8"):
        M = inputs[name]
        Mt = G.transpose(M)
        for sr in (O.SR_PLUSTIMES_F64, O.SR_PLUSTIMES_F32, O.SR_PLUSTIMES_I64, O.SR_MINPLUS_F64,
                   O.SR_SELECT2NDMIN_I64, O.SR_BOOL, O.SR_MINPLUS_I64):
            A = with_type(M, sr, 1)
            At = with_type(Mt, sr, 2)
            put_prod(d, f"prod/{name}/AA/{sr}", A, A, sr)
            put_prod(d, f"prod/{name}/AAt/{sr}", A, At, sr)
            cases.append(name)
        # the hash-only variants (sorted and unsorted row order)
        A = with_type(M, O.SR_PLUSTIMES_F64, 1)
        put_prod(d, f"prod/{name}/AA_hash_sorted/0", A, A, O.SR_PLUSTIMES_F64, O.V_HASH_SORTED)
        put_prod(d, f"prod/{name}/AA_hash_unsorted/0", A, A, O.SR_PLUSTIMES_F64, O.V_HASH_UNSORTED)
        put_prod(d, f"prod/{name}/AA_heap/0", A, A, O.SR_PLUSTIMES_F64, O.V_HEAP)
        put_prod(d, f"prod/{name}/AA_pspgemm/0", A, A, O.SR_PLUSTIMES_F64, O.V_PSPGEMM)
        d[f"colstats/{name}/flop"] = O.ref_colstats(M, M, 0)
        d[f"colstats/{name}/nnz"] = O.ref_colstats(M, M, 1)
    # DCSC input with empty columns: A (300x260) times a 260x120 random B
    B = G.random_sparse(260, 120, 0.05, seed=6, empty_cols=0.25)
    put_mat(d, "in/rand_dcsc_B", B)
    for sr in (O.SR_PLUSTIMES_F64, O.SR_SELECT2NDMIN_I64, O.SR_BOOL):
        put_prod(d, f"prod/rand_dcsc/AB/{sr}", with_type(rm_dcsc, sr, 3), with_type(B, sr, 4), sr)
    # BFS (min-parent SpMSpV loop) on symmetric patterns
    for name in ("seven_sym", "torus", "rmat8"):
        M = inputs["seven"] if name == "seven_sym" else inputs[name]
        if name == "seven_sym":
            T = G.transpose(M)
            rows = np.concatenate([M.rowidx, T.rowidx])
            cols = np.concatenate([M.col_ids(), T.col_ids()])
            keep = rows != cols
            M = G.csc_from_coo(M.nrow, M.ncol, rows[keep], cols[keep])
            put_mat(d, "in/seven_sym", M)
        P = M.with_values(None)
        srcs = [0, 1, M.ncol // 2, M.ncol - 1]
        d[f"bfs/{name}/sources"] = np.array(srcs, np.int64)
        for s in srcs:
            par, lev, it, _ = O.ref_bfs(P, s)
            d[f"bfs/{name}/{s}/parents"] = par
            d[f"bfs/{name}/{s}/levels"] = lev
            d[f"bfs/{name}/{s}/iters"] = np.array(it)
    # one SpMSpV (bucket algorithm) on rmat8
    rng = np.random.default_rng(9)
    x = np.sort(rng.choice(rm.ncol, 40, replace=False)).astype(np.int32)
    xv = rng.integers(0, rm.ncol, 40).astype(np.int64)
    yr, yv = O.ref_spmspv(rm.with_values(None), x, xv)
    d["spmspv/rmat8/x_ind"] = x
    d["spmspv/rmat8/x_val"] = xv
    d["spmspv/rmat8/y_ind"] = yr
    d["spmspv/rmat8/y_val"] = yv
    # the other SpMXSpV semirings on a rectangular 1500 x 1000 matrix
    rng = np.random.default_rng(12)
    R = G.csc_from_coo(1500, 1000, rng.integers(0, 1500, 12000), rng.integers(0, 1000, 12000),
                       rng.random(12000) * 2 - 1)
    put_mat(d, "in/rect1500", R)
    x = np.sort(rng.choice(1000, 120, replace=False)).astype(np.int32)
    d["spmspvsr/x_ind"] = x
    d["spmspvsr/x_i64"] = rng.integers(-1000, 1000, 120).astype(np.int64)
    d["spmspvsr/x_f64"] = rng.random(120) * 2 - 1
    for sx in (O.SX_SELECT2ND, O.SX_SELECTMAX):
        d[f"spmspvsr/{sx}/y_ind"], d[f"spmspvsr/{sx}/y_val"] = O.ref_spmspv_sr(R, sx, x, d["spmspvsr/x_i64"])
    for dt in (np.float64, np.float32):
        d[f"spmspvsr/3/{np.dtype(dt).name}/y_ind"], d[f"spmspvsr/3/{np.dtype(dt).name}/y_val"] = O.ref_spmspv_sr(
            R.with_values(R.values.astype(dt)), O.SX_PLUSTIMES, x, d["spmspvsr/x_f64"].astype(dt), dt)
    Ri = R.with_values(np.round(R.values * 100).astype(np.int64))
    d["spmspvsr/3/int64/y_ind"], d["spmspvsr/3/int64/y_val"] = O.ref_spmspv_sr(Ri, O.SX_PLUSTIMES, x,
                                                                                d["spmspvsr/x_i64"], np.int64)
    # multi-source BFS (MD.cpp's Select2ndMin SpGEMM loop) on rmat8 and torus
    for name, Mm in (("rmat8", rm), ("torus", torus)):
        P = Mm.with_values(None)
        deg = np.diff(P.colptr)
        roots = np.random.default_rng(11).choice(np.nonzero(deg)[0], 12, replace=False).astype(np.int64)
        par, lv = O.ref_msbfs(P, roots)
        d[f"msbfs/{name}/roots"] = roots
        d[f"msbfs/{name}/parents"] = par
        d[f"msbfs/{name}/levels"] = np.array(lv)
    # MultiwayMerge of overlapping lists (several SUMMA stages of one block)
    base = G.random_sparse(400, 250, 0.04, seed=21)
    rng = np.random.default_rng(22)
    lists = [G.random_sparse(400, 250, 0.02, seed=30 + k) for k in range(3)]
    lists = [base.with_values((1.0 - rng.random(base.nnz)) * 10.0 ** rng.integers(-6, 6, base.nnz))] + \
        [M.with_values(1.0 - rng.random(M.nnz)) for M in lists]
    for k, M in enumerate(lists):
        put_mat(d, f"in/merge{k}", M)
    for K in (2, 4):
        for sr in (O.SR_PLUSTIMES_F64, O.SR_SELECT2NDMIN_I64):
            L = [with_type(M, sr, 40 + k) if sr != O.SR_PLUSTIMES_F64 else M for k, M in enumerate(lists[:K])]
            r, c, v = O.ref_multiway_merge(L, 400, 250, sr)
            key = f"merge/{K}/{sr}"
            d[f"{key}/rows"], d[f"{key}/cols"], d[f"{key}/vals"] = r, c, v
    # dcsc_gespmv: y <- y (+) A x on rmat8
    rng = np.random.default_rng(23)
    for sr in (O.SR_PLUSTIMES_F64, O.SR_MINPLUS_F64, O.SR_SELECT2NDMIN_I64, O.SR_BOOL):
        Mt = with_type(rm, sr, 50 + sr)
        dt = O.SR_DTYPE[sr]
        if dt == np.bool_:
            x, y = rng.random(rm.ncol) < 0.5, rng.random(rm.nrow) < 0.2
        elif dt == np.int64:
            x, y = rng.integers(0, 100, rm.ncol), rng.integers(0, 200, rm.nrow)
        else:
            x, y = rng.random(rm.ncol), rng.random(rm.nrow) * 3
        d[f"spmv/{sr}/x"], d[f"spmv/{sr}/y0"] = x, y
        d[f"spmv/{sr}/y"] = O.ref_spmv(Mt, x, y, sr)
    # MCL expansion + prune/select
    M = G.mcl_planted(4096, 256, 10, 3, seed=5)
    put_mat(d, "in/mcl4096", M)
    for thr, k in ((1e-4, 30), (1e-3, 12)):
        r, c, v, _ = O.ref_mcl_expand(M, thr, k)
        key = f"mcl/mcl4096/{thr:g}/{k}"
        d[f"{key}/rows"] = r
        d[f"{key}/cols"] = c
        d[f"{key}/vals"] = v
    # MCL prune/select with recovery (ParFriends.h:290-330)
    for thr, k, rn, pct in ((1e-2, 30, 40, 0.9), (5e-3, 20, 30, 0.95), (2e-2, 10, 25, 0.8), (3e-2, 5, 12, 0.9)):
        r, c, v, _ = O.ref_mcl_expand(M, thr, k, rn, pct)
        key = f"mclrec/mcl4096/{thr:g}/{k}/{rn}/{pct:g}"
        d[f"{key}/rows"] = r
        d[f"{key}/cols"] = c
        d[f"{key}/vals"] = v
    # MCL vector steps (MCL.cpp:389-449) and the HipMCL loop (:526-626)
    (cp, r, v), _, _ = O.ref_mcl_iterate(M, mode=1)
    d["mclstep/mcl4096/colscale"] = v
    for power in (2.0, 1.5):
        (cp, r, v), _, _ = O.ref_mcl_iterate(M, inflation=power, mode=2)
        d[f"mclstep/mcl4096/inflate/{power:g}"] = v
    _, _, chaos = O.ref_mcl_iterate(M, mode=3)
    d["mclstep/mcl4096/chaos"] = np.array([chaos], np.float32)
    for infl, thr, k, rn, pct, mi in ((2.0, 1e-4, 30, 40, 0.9, 0), (1.5, 1e-3, 20, 30, 0.9, 0),
                                      (2.0, 1e-4, 30, 40, 0.9, 2)):
        (cp, r, v), it, chaos = O.ref_mcl_iterate(M, infl, thr, k, rn, pct, mi)
        key = f"mclloop/mcl4096/{infl:g}/{thr:g}/{k}/{rn}/{pct:g}/{mi}"
        d[f"{key}/colptr"] = cp
        d[f"{key}/rowidx"] = r
        d[f"{key}/values"] = v
        d[f"{key}/iterations"] = np.array([it], np.int64)
        d[f"{key}/chaos"] = np.array([chaos], np.float32)
    # Galerkin triple product R * (A * R^T) on a 4^3 Poisson grid
    A = G.poisson27(4)
    R = G.aggregation(4)
    Rt = G.transpose(R)
    put_mat(d, "in/poisson4", A)
    put_mat(d, "in/agg4", R)
    r, c, v, _ = O.ref_spgemm(A, Rt, O.SR_PLUSTIMES_F64)
    AR = O.tuples_to_csc(r, c, v, Rt.ncol)
    ARm = G.CSC(A.nrow, Rt.ncol, AR[0], AR[1], AR[2])
    put_prod(d, "prod/galerkin4/RAR/0", R, ARm, O.SR_PLUSTIMES_F64)
    np.savez_compressed(OUT, **d)
    print(f"wrote {OUT}: {len(d)} arrays, {os.path.getsize(OUT)} bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("COMBBLAS_REF", "/root/reference"))
