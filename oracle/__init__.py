"""Oracle: test infrastructure, never product code.

Two CPU implementations of the local SpGEMM / SpMSpV / MCL-select path are
reachable from here, both used only as checkers by ``tests/``, by
``__graft_entry__.smoke()`` and by the CPU-baseline leg of ``bench.py``:

* ``port`` -- the project's own plain-C restatement of the reference's
  algorithms (``oracle/oracle.c``), built everywhere by ``oracle/Makefile``;
* ``ref``  -- the reference's own header templates compiled unchanged against
  a single-rank MPI stand-in (``oracle/ref_harness.cpp``); it only exists where
  the reference sources were present at build time.

The product (``combblas_gb300``) never imports this package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REF_SO = os.path.join(_HERE, "_ref", "libcombblas_ref.so")
_PORT_SO = os.path.join(_HERE, "_ref", "libgbc_oracle.so")

# semiring codes shared by both libraries
SR_PLUSTIMES_F64 = 0
SR_PLUSTIMES_F32 = 1
SR_PLUSTIMES_I64 = 2
SR_MINPLUS_F64 = 3
SR_SELECT2NDMIN_I64 = 4
SR_BOOL = 5
SR_MINPLUS_I64 = 6

SR_DTYPE = {
    SR_PLUSTIMES_F64: np.float64,
    SR_PLUSTIMES_F32: np.float32,
    SR_PLUSTIMES_I64: np.int64,
    SR_MINPLUS_F64: np.float64,
    SR_SELECT2NDMIN_I64: np.int64,
    SR_BOOL: np.bool_,
    SR_MINPLUS_I64: np.int64,
}

# variant codes of ref_spgemm
V_HYBRID = 0
V_HEAP = 1
V_HASH_SORTED = 2
V_HASH_UNSORTED = 3
V_HYBRID_CSC = 4
V_PSPGEMM = 5

_P64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_P32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(ref_path: str | None = None, quiet: bool = True) -> None:
    """Compile the oracle libraries in place (``make -C oracle``)."""
    import subprocess

    cmd = ["make", "-C", _HERE, "-j4"]
    if ref_path:
        cmd.append(f"REF={ref_path}")
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL if quiet else None)


def have_ref() -> bool:
    return os.path.exists(_REF_SO)


_ref_lib = None
_port_lib = None


def _ref():
    global _ref_lib
    if _ref_lib is None:
        lib = C.CDLL(_REF_SO)
        lib.ref_spgemm.restype = C.c_int64
        lib.ref_spgemm.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_int64, _P64, _P64, C.c_void_p,
                                   _P64, _P64, C.c_void_p, C.c_int]
        lib.ref_result_copy.restype = None
        lib.ref_result_copy.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ref_result_seconds.restype = C.c_double
        lib.ref_colstats.restype = C.c_int64
        lib.ref_colstats.argtypes = [C.c_int, C.c_int64, C.c_int64, C.c_int64, _P64, _P64, _P64, _P64, _P64]
        lib.ref_spmspv_bucket.restype = C.c_int64
        lib.ref_spmspv_bucket.argtypes = [C.c_int64, C.c_int64, _P64, _P64, _P32, _P64, C.c_int32, C.c_int]
        lib.ref_bfs_selectmin.restype = C.c_int
        lib.ref_bfs_selectmin.argtypes = [C.c_int64, _P64, _P64, C.c_int64, _P64, C.c_void_p]
        lib.ref_mcl_expand.restype = C.c_int64
        lib.ref_mcl_expand.argtypes = [C.c_int64, _P64, _P64, np.ctypeslib.ndpointer(dtype=np.float32),
                                       C.c_float, C.c_int64, C.c_int64, C.c_float]
        lib.ref_num_threads.restype = C.c_int
        lib.ref_result_nnz.restype = C.c_int64
        lib.ref_spmspv_sr.restype = C.c_int64
        lib.ref_spmspv_sr.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_int64, _P64, _P64, C.c_void_p, _P32,
                                      C.c_void_p, C.c_int32]
        lib.ref_mcl_iterate.restype = C.c_int64
        lib.ref_mcl_iterate.argtypes = [C.c_int64, _P64, _P64, np.ctypeslib.ndpointer(dtype=np.float32), C.c_double,
                                        C.c_float, C.c_int64, C.c_int64, C.c_float, C.c_int64, C.c_int,
                                        C.POINTER(C.c_float)]
        lib.ref_spmv.restype = C.c_int
        lib.ref_spmv.argtypes = [C.c_int, C.c_int64, C.c_int64, _P64, _P64, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ref_multiway_merge.restype = C.c_int64
        lib.ref_multiway_merge.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                           C.c_void_p]
        _ref_lib = lib
    return _ref_lib


def _vals_ptr(M, dtype):
    if M.values is None:
        return None, None
    v = np.ascontiguousarray(M.values, dtype=dtype)
    return v, v.ctypes.data_as(C.c_void_p)


def _fetch(lib, nnz, dtype, with_cols=True):
    rows = np.empty(nnz, np.int64)
    cols = np.empty(nnz, np.int64) if with_cols else None
    vals = np.empty(nnz, dtype)
    lib.ref_result_copy(rows.ctypes.data_as(C.c_void_p),
                        cols.ctypes.data_as(C.c_void_p) if with_cols else None,
                        vals.ctypes.data_as(C.c_void_p))
    return rows, cols, vals


# ------------------------------------------------------------------ reference
def ref_spgemm(A, B, sr: int, variant: int = V_HYBRID, reps: int = 1):
    """Run the reference's own local multiply.  Returns (rows, cols, vals,
    seconds) in the order the reference emits them (SpTuples order)."""
    lib = _ref()
    dt = SR_DTYPE[sr]
    av, ap = _vals_ptr(A, dt)
    bv, bp = _vals_ptr(B, dt)
    nnz = lib.ref_spgemm(variant, sr, A.nrow, A.ncol, B.ncol, np.ascontiguousarray(A.colptr),
                         np.ascontiguousarray(A.rowidx), ap, np.ascontiguousarray(B.colptr),
                         np.ascontiguousarray(B.rowidx), bp, reps)
    if nnz < 0:
        raise ValueError("bad semiring/variant")
    rows, cols, vals = _fetch(lib, nnz, dt)
    return rows, cols, vals, lib.ref_result_seconds()


def ref_colstats(A, B, which: int):
    """Per nonempty column of B: 0 = estimateFLOP, 1 = estimateNNZ_Hash."""
    lib = _ref()
    out = np.zeros(max(B.ncol, 1), np.int64)
    nzc = lib.ref_colstats(which, A.nrow, A.ncol, B.ncol, np.ascontiguousarray(A.colptr),
                           np.ascontiguousarray(A.rowidx), np.ascontiguousarray(B.colptr),
                           np.ascontiguousarray(B.rowidx), out)
    return out[:nzc]


def ref_spmspv(A, indx: np.ndarray, numx: np.ndarray, buckets: int = 32):
    lib = _ref()
    indx = np.ascontiguousarray(indx, np.int32)
    numx = np.ascontiguousarray(numx, np.int64)
    nnz = lib.ref_spmspv_bucket(A.nrow, A.ncol, np.ascontiguousarray(A.colptr), np.ascontiguousarray(A.rowidx),
                                indx, numx, len(indx), buckets)
    rows, _, vals = _fetch(lib, nnz, np.int64, with_cols=False)
    return rows, vals


def ref_bfs(A, source: int, with_levels: bool = True):
    lib = _ref()
    n = A.ncol
    parents = np.empty(n, np.int64)
    levels = np.empty(n, np.int64) if with_levels else None
    it = lib.ref_bfs_selectmin(n, np.ascontiguousarray(A.colptr), np.ascontiguousarray(A.rowidx), int(source),
                               parents, levels.ctypes.data_as(C.c_void_p) if with_levels else None)
    return parents, levels, it, lib.ref_result_seconds()


def ref_mcl_expand(A, thr: float, select: int, recover_num: int = 0, recover_pct: float = 0.9):
    lib = _ref()
    nnz = lib.ref_mcl_expand(A.ncol, np.ascontiguousarray(A.colptr), np.ascontiguousarray(A.rowidx),
                             np.ascontiguousarray(A.values, np.float32), thr, select, recover_num, recover_pct)
    rows, cols, vals = _fetch(lib, nnz, np.float32)
    return rows, cols, vals, lib.ref_result_seconds()


def ref_mcl_iterate(A, inflation: float = 2.0, thr: float = 1e-4, select: int = 1100, recover_num: int = 1400,
                    recover_pct: float = 0.9, max_iter: int = 0, mode: int = 0):
    """The HipMCL loop (mode 0) or one of its vector steps (1 MakeColStochastic,
    2 Inflate, 3 Chaos) run by the reference's own SpParMat calls
    (ref_harness.cpp ref_mcl_iterate).  Returns (canonical CSC, iterations,
    chaos)."""
    lib = _ref()
    chaos = C.c_float(0.0)
    it = lib.ref_mcl_iterate(A.ncol, np.ascontiguousarray(A.colptr), np.ascontiguousarray(A.rowidx),
                             np.ascontiguousarray(A.values, np.float32), float(inflation), float(thr), int(select),
                             int(recover_num), float(recover_pct), int(max_iter), int(mode), C.byref(chaos))
    rows, cols, vals = _fetch(lib, lib.ref_result_nnz(), np.float32)
    return tuples_to_csc(rows, cols, vals, A.ncol), it, chaos.value


def ref_num_threads() -> int:
    return _ref().ref_num_threads()


# ----------------------------------------------------------------------- port
def _port():
    global _port_lib
    if _port_lib is None:
        lib = C.CDLL(_PORT_SO)
        lib.gbc_o_spgemm.restype = C.c_int64
        lib.gbc_o_spgemm.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_int64, _P64, _P64, C.c_void_p,
                                     _P64, _P64, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.gbc_o_spgemm_exact.restype = C.c_int64
        lib.gbc_o_spgemm_exact.argtypes = [C.c_int64, C.c_int64, C.c_int64, _P64, _P64, C.c_void_p, _P64, _P64,
                                           C.c_void_p, C.c_void_p, C.c_void_p]
        lib.gbc_o_result.restype = None
        lib.gbc_o_result.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.gbc_o_spmspv.restype = C.c_int64
        lib.gbc_o_spmspv.argtypes = [C.c_int64, _P64, _P64, _P32, _P64, C.c_int32, C.c_int]
        lib.gbc_o_spmspv_sr.restype = C.c_int64
        lib.gbc_o_spmspv_sr.argtypes = [C.c_int, C.c_int, C.c_int64, _P64, _P64, C.c_void_p, _P32, C.c_void_p,
                                        C.c_int32]
        lib.gbc_o_bfs.restype = C.c_int
        lib.gbc_o_bfs.argtypes = [C.c_int64, _P64, _P64, C.c_int64, _P64, C.c_void_p]
        lib.gbc_o_mcl_select.restype = C.c_int64
        lib.gbc_o_mcl_select.argtypes = [C.c_int64, _P64, _P64, np.ctypeslib.ndpointer(dtype=np.float32),
                                         C.c_float, C.c_int64]
        lib.gbc_o_mcl_select_recover.restype = C.c_int64
        lib.gbc_o_mcl_select_recover.argtypes = [C.c_int64, _P64, _P64, np.ctypeslib.ndpointer(dtype=np.float32),
                                                 C.c_float, C.c_int64, C.c_int64, C.c_float]
        lib.gbc_o_mcl_colscale.restype = None
        lib.gbc_o_mcl_colscale.argtypes = [C.c_int64, _P64, np.ctypeslib.ndpointer(dtype=np.float32)]
        lib.gbc_o_mcl_chaos.restype = C.c_float
        lib.gbc_o_mcl_chaos.argtypes = [C.c_int64, _P64, np.ctypeslib.ndpointer(dtype=np.float32)]
        lib.gbc_o_mcl_inflate.restype = None
        lib.gbc_o_mcl_inflate.argtypes = [C.c_int64, np.ctypeslib.ndpointer(dtype=np.float32), C.c_double]
        lib.gbc_o_num_threads.restype = C.c_int
        _port_lib = lib
    return _port_lib


def _port_csc(lib, ncol, nnz, dtype):
    cp = np.empty(ncol + 1, np.int64)
    rows = np.empty(nnz, np.int64)
    vals = np.empty(nnz, dtype)
    lib.gbc_o_result(cp.ctypes.data_as(C.c_void_p), rows.ctypes.data_as(C.c_void_p),
                     vals.ctypes.data_as(C.c_void_p))
    return cp, rows, vals


def port_spgemm(A, B, sr: int, sorted: bool = True, want_counts: bool = False, fold: str = "ordered"):
    """C = A*B by the C restatement.  Returns a CSC (generators.CSC-like
    tuple: colptr, rowidx, values) and optionally (flop, nnz) per column.
    fold="exact" (PlusTimes fp64 only): the library's exact fold -- each
    entry the exact sum of the rounded products, rounded once (rows sorted)."""
    lib = _port()
    dt = SR_DTYPE[sr]
    av, ap = _vals_ptr(A, dt)
    bv, bp = _vals_ptr(B, dt)
    if ap is None:
        av = np.ones(A.nnz, dt)
        ap = av.ctypes.data_as(C.c_void_p)
    if bp is None:
        bv = np.ones(B.nnz, dt)
        bp = bv.ctypes.data_as(C.c_void_p)
    flop = np.empty(B.ncol, np.int64)
    cnt = np.empty(B.ncol, np.int64)
    if fold == "exact":
        if sr != SR_PLUSTIMES_F64:
            raise ValueError("the exact fold is defined for PlusTimes fp64")
        nnz = lib.gbc_o_spgemm_exact(A.nrow, A.ncol, B.ncol, np.ascontiguousarray(A.colptr),
                                     np.ascontiguousarray(A.rowidx), ap, np.ascontiguousarray(B.colptr),
                                     np.ascontiguousarray(B.rowidx), bp, flop.ctypes.data_as(C.c_void_p),
                                     cnt.ctypes.data_as(C.c_void_p))
    else:
        nnz = lib.gbc_o_spgemm(sr, int(sorted), A.nrow, A.ncol, B.ncol, np.ascontiguousarray(A.colptr),
                               np.ascontiguousarray(A.rowidx), ap, np.ascontiguousarray(B.colptr),
                               np.ascontiguousarray(B.rowidx), bp, flop.ctypes.data_as(C.c_void_p),
                               cnt.ctypes.data_as(C.c_void_p))
    if nnz < 0:
        raise ValueError("bad semiring")
    cp, rows, vals = _port_csc(lib, B.ncol, nnz, dt)
    if want_counts:
        return (cp, rows, vals), (flop, cnt)
    return cp, rows, vals


# SpMSpV semiring codes of ref_spmspv_sr / gbc_o_spmspv_sr
SX_SELECTMIN, SX_SELECT2ND, SX_SELECTMAX, SX_PLUSTIMES = 0, 1, 2, 3
_SX_VT = {np.float64: 0, np.float32: 1, np.int64: 2}


def _sx_args(A, sx, indx, numx, dtype):
    dt = np.int64 if sx != SX_PLUSTIMES else dtype
    indx = np.ascontiguousarray(indx, np.int32)
    numx = np.ascontiguousarray(numx, dt)
    av = None
    if sx == SX_PLUSTIMES:
        av = np.ascontiguousarray(A.values if A.values is not None else np.ones(A.nnz), dt)
    return dt, indx, numx, av


def ref_spmspv_sr(A, sx: int, indx, numx, dtype=np.float64):
    """The reference's own SpMXSpV over Select2nd (boolean optbuf path),
    SelectMax or PlusTimes (SpMXSpV_Bucket).  Returns (rows, values)."""
    lib = _ref()
    dt, indx, numx, av = _sx_args(A, sx, indx, numx, dtype)
    ny = lib.ref_spmspv_sr(sx, _SX_VT.get(dt, 2), A.nrow, A.ncol, np.ascontiguousarray(A.colptr),
                           np.ascontiguousarray(A.rowidx), None if av is None else av.ctypes.data_as(C.c_void_p),
                           indx, numx.ctypes.data_as(C.c_void_p), len(indx))
    if ny < 0:
        raise ValueError("bad semiring")
    rows, _, vals = _fetch(lib, ny, dt, with_cols=False)
    return rows, vals


def port_spmspv_sr(A, sx: int, indx, numx, dtype=np.float64):
    """The restatement (oracle.c gbc_o_spmspv_sr).  Returns (rows, values)."""
    lib = _port()
    dt, indx, numx, av = _sx_args(A, sx, indx, numx, dtype)
    ny = lib.gbc_o_spmspv_sr(sx, _SX_VT.get(dt, 2), A.nrow, np.ascontiguousarray(A.colptr),
                             np.ascontiguousarray(A.rowidx), None if av is None else av.ctypes.data_as(C.c_void_p),
                             indx, numx.ctypes.data_as(C.c_void_p), len(indx))
    rows = np.empty(ny, np.int64)
    vals = np.empty(ny, dt)
    lib.gbc_o_result(None, rows.ctypes.data_as(C.c_void_p), vals.ctypes.data_as(C.c_void_p))
    return rows, vals


def port_spmspv(A, indx, numx, buckets: int = 32):
    lib = _port()
    indx = np.ascontiguousarray(indx, np.int32)
    numx = np.ascontiguousarray(numx, np.int64)
    ny = lib.gbc_o_spmspv(A.nrow, np.ascontiguousarray(A.colptr), np.ascontiguousarray(A.rowidx), indx, numx,
                          len(indx), buckets)
    rows = np.empty(ny, np.int64)
    vals = np.empty(ny, np.int64)
    lib.gbc_o_result(None, rows.ctypes.data_as(C.c_void_p), vals.ctypes.data_as(C.c_void_p))
    return rows, vals


def port_bfs(A, source: int, with_levels: bool = True):
    lib = _port()
    n = A.ncol
    parents = np.empty(n, np.int64)
    levels = np.empty(n, np.int64) if with_levels else None
    it = lib.gbc_o_bfs(n, np.ascontiguousarray(A.colptr), np.ascontiguousarray(A.rowidx), int(source), parents,
                       levels.ctypes.data_as(C.c_void_p) if with_levels else None)
    return parents, levels, it


def ref_multiway_merge(lists, m: int, n: int, sr: int):
    """The reference's MultiwayMerge<SR> of CSC matrices of one shape;
    returns (rows, cols, vals) in its column-major tuple order."""
    lib = _ref()
    dt = SR_DTYPE[sr]
    keep = []
    cps = (C.c_void_p * max(len(lists), 1))()
    ris = (C.c_void_p * max(len(lists), 1))()
    vls = (C.c_void_p * max(len(lists), 1))()
    for k, M in enumerate(lists):
        cp = np.ascontiguousarray(M.colptr, np.int64)
        ri = np.ascontiguousarray(M.rowidx, np.int64)
        v = np.ascontiguousarray(M.values, dt) if M.values is not None else np.ones(len(ri), dt)
        keep += [cp, ri, v]
        cps[k], ris[k], vls[k] = cp.ctypes.data, ri.ctypes.data, v.ctypes.data
    nnz = lib.ref_multiway_merge(sr, len(lists), m, n, cps, ris, vls)
    if nnz < 0:
        raise ValueError("bad semiring")
    return _fetch(lib, nnz, dt)


def _sr_add(sr: int, a, b):
    if sr in (SR_MINPLUS_F64, SR_MINPLUS_I64, SR_SELECT2NDMIN_I64):
        return np.where(b < a, b, a)  # std::min(a, b)
    if sr == SR_BOOL:
        return np.logical_or(a, b)
    return a + b  # IEEE / wrap-around, as the reference's add


def port_multiway_merge(lists, m: int, n: int, sr: int):
    """Restatement of MultiwayMerge (MultiwayMerge.h:193-240 SerialMerge):
    entries of all lists in column-major order, equal (row, col) combined
    by SR::add in list order.  Returns a CSC (colptr, rows, vals)."""
    dt = SR_DTYPE[sr]
    rows, cols, vals, src = [], [], [], []
    for k, M in enumerate(lists):
        cnt = np.diff(M.colptr)
        rows.append(np.asarray(M.rowidx, np.int64))
        cols.append(np.repeat(np.arange(n, dtype=np.int64), cnt))
        vals.append(np.asarray(M.values, dt) if M.values is not None else np.ones(int(M.colptr[-1]), dt))
        src.append(np.full(int(M.colptr[-1]), k, np.int64))
    if not lists:
        return np.zeros(n + 1, np.int64), np.zeros(0, np.int64), np.zeros(0, dt)
    r, c, v, k = (np.concatenate(x) for x in (rows, cols, vals, src))
    order = np.lexsort((k, r, c))
    r, c, v = r[order], c[order], v[order]
    key = c * m + r
    start = np.ones(len(key), bool)
    start[1:] = key[1:] != key[:-1]
    head = np.nonzero(start)[0]
    run = np.cumsum(start) - 1
    occ = np.arange(len(key)) - head[run]
    acc = v[head].copy()
    for level in range(1, int(occ.max(initial=0)) + 1):
        sel = occ == level
        acc[run[sel]] = _sr_add(sr, acc[run[sel]], v[sel])
    rr, cc = r[head], c[head]
    colptr = np.zeros(n + 1, np.int64)
    colptr[1:] = np.cumsum(np.bincount(cc, minlength=n))
    return colptr, rr, acc.astype(dt)


def ref_spmv(A, x, y, sr: int):
    """The reference's dcsc_gespmv<SR>: returns y (+) A x (y is copied)."""
    lib = _ref()
    dt = SR_DTYPE[sr]
    v = np.ascontiguousarray(A.values, dt) if A.values is not None else np.ones(A.nnz, dt)
    x = np.ascontiguousarray(x, dt)
    y = np.array(y, dt)
    if lib.ref_spmv(sr, A.nrow, A.ncol, np.ascontiguousarray(A.colptr), np.ascontiguousarray(A.rowidx),
                    v.ctypes.data, x.ctypes.data, y.ctypes.data) != 0:
        raise ValueError("bad semiring")
    return y


def port_spmv(A, x, y, sr: int):
    """Restatement of dcsc_gespmv (Friends.h:63-77): for every column in
    order, for its entries, y[row] = axpy(a, x[col], y[row]); returns a copy."""
    dt = SR_DTYPE[sr]
    y = np.array(y, dt)
    x = np.asarray(x, dt)
    v = np.asarray(A.values, dt) if A.values is not None else np.ones(A.nnz, dt)
    for j in range(A.ncol):
        s0, s1 = int(A.colptr[j]), int(A.colptr[j + 1])
        if s0 == s1:
            continue
        r = A.rowidx[s0:s1]
        a = v[s0:s1]
        if sr in (SR_PLUSTIMES_F64, SR_PLUSTIMES_F32, SR_PLUSTIMES_I64):
            y[r] = y[r] + a * x[j]
        elif sr == SR_BOOL:
            y[r] = np.logical_or(y[r], np.logical_and(a, x[j]))
        elif sr in (SR_MINPLUS_F64, SR_MINPLUS_I64):
            inf = np.finfo(dt).max if dt == np.float64 else np.iinfo(dt).max
            t = np.where((a == inf) | (x[j] == inf), inf, a + x[j])
            y[r] = np.where(t < y[r], t, y[r])
        else:  # Select2ndMin: multiply returns x
            y[r] = np.where(x[j] < y[r], x[j], y[r])
    return y


def msbfs_loop(A, roots, multiply):
    """Multi-source BFS as the reference's Select2ndMin SpGEMM loop
    (Applications/Ordering/MD.cpp:200-217): F starts with F(root_r, r) =
    root_r and visited = the sources; each level F = multiply(A, F) (a
    Select2ndMin product returning a CSC), then EWiseMult(F, visited,
    exclude=true), visited += F, and every value becomes its own row id.
    parents[r, v] = the product's value when v entered; parents[r, root_r]
    = root_r; -1 if never reached.  Returns (parents, levels)."""
    n = A.ncol
    R = len(roots)
    roots = np.asarray(roots, np.int64)
    parents = np.full((R, n), -1, np.int64)
    visited = np.zeros((R, n), bool)
    visited[np.arange(R), roots] = True
    parents[np.arange(R), roots] = roots

    class _F:
        pass

    F = _F()
    F.nrow, F.ncol = n, R
    F.colptr = np.arange(R + 1, dtype=np.int64)
    F.rowidx = roots.copy()
    F.values = roots.copy()
    levels = 0
    while F.rowidx.size:
        cp, rows, vals = multiply(A, F)
        cols = np.repeat(np.arange(R, dtype=np.int64), np.diff(cp))
        keep = ~visited[cols, rows]
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
        visited[cols, rows] = True
        parents[cols, rows] = vals
        F = _F()
        F.nrow, F.ncol = n, R
        F.colptr = np.zeros(R + 1, np.int64)
        F.colptr[1:] = np.cumsum(np.bincount(cols, minlength=R))
        F.rowidx = rows.astype(np.int64)
        F.values = rows.astype(np.int64)
        levels += 1
    return parents, levels


def port_msbfs(A, roots):
    """msbfs_loop over the C restatement's Select2ndMin product."""
    Ap = A.with_values(np.ones(A.nnz, np.int64))
    return msbfs_loop(Ap, roots, lambda X, F: port_spgemm(X, F, SR_SELECT2NDMIN_I64))


def ref_msbfs(A, roots):
    """msbfs_loop over the reference's own PSpGEMM<Select2ndMinSR> on a 1x1 grid."""
    Ap = A.with_values(np.ones(A.nnz, np.int64))

    def mult(X, F):
        r, c, v, _ = ref_spgemm(X, F, SR_SELECT2NDMIN_I64, V_PSPGEMM)
        return tuples_to_csc(r, c, v, F.ncol)

    return msbfs_loop(Ap, roots, mult)


def port_mcl_select(Ccp, Cri, Cv, thr: float, select: int, recover_num: int = 0, recover_pct: float = 0.0):
    """MCLPruneRecoverySelect restated (oracle.c gbc_o_mcl_select_recover)."""
    lib = _port()
    n = len(Ccp) - 1
    nnz = lib.gbc_o_mcl_select_recover(n, np.ascontiguousarray(Ccp, np.int64), np.ascontiguousarray(Cri, np.int64),
                                       np.ascontiguousarray(Cv, np.float32), thr, select, recover_num, recover_pct)
    return _port_csc(lib, n, nnz, np.float32)


def port_mcl_colscale(cp, v):
    """MakeColStochastic restated (oracle.c gbc_o_mcl_colscale); new values."""
    v = np.array(v, np.float32)
    _port().gbc_o_mcl_colscale(len(cp) - 1, np.ascontiguousarray(cp, np.int64), v)
    return v


def port_mcl_chaos(cp, v) -> float:
    """Chaos restated (oracle.c gbc_o_mcl_chaos)."""
    return _port().gbc_o_mcl_chaos(len(cp) - 1, np.ascontiguousarray(cp, np.int64), np.ascontiguousarray(v, np.float32))


def port_mcl_inflate(v, power: float):
    """Inflate restated (oracle.c gbc_o_mcl_inflate); new values."""
    v = np.array(v, np.float32)
    _port().gbc_o_mcl_inflate(len(v), v, float(power))
    return v


class _Csc:
    def __init__(self, n, cp, ri, v):
        self.nrow = self.ncol = n
        self.colptr, self.rowidx, self.values = cp, ri, v
        self.nnz = len(ri)


def port_mcl_iterate(A, inflation: float = 2.0, thr: float = 1e-4, select: int = 1100, recover_num: int = 1400,
                     recover_pct: float = 0.9, max_iter: int = 0):
    """The HipMCL loop of Applications/MCL.cpp:526-626 (one layer, one phase)
    restated over the port's SpGEMM, prune/select/recovery and vector steps:
    MakeColStochastic, the pre-loop prune when nnz / n > max(select,
    recover_num), then while chaos > 0.0001 (EPS, :55): expand + prune,
    MakeColStochastic, Chaos, Inflate, MakeColStochastic.  Returns
    (canonical CSC, iterations, chaos)."""
    n = A.ncol
    cp, ri = np.asarray(A.colptr, np.int64), np.asarray(A.rowidx, np.int64)
    v = port_mcl_colscale(cp, A.values)
    if n > 0 and len(ri) // n > max(select, recover_num):
        cp, ri, v = port_mcl_select(cp, ri, v, thr, select, recover_num, recover_pct)
    chaos, it = np.float32(1.0), 0
    while float(chaos) > 0.0001 and (max_iter <= 0 or it < max_iter):
        M = _Csc(n, cp, ri, v)
        pcp, pri, pv = port_spgemm(M, M, SR_PLUSTIMES_F32, sorted=True)
        cp, ri, v = port_mcl_select(pcp, pri, pv, thr, select, recover_num, recover_pct)
        v = port_mcl_colscale(cp, v)
        chaos = np.float32(port_mcl_chaos(cp, v))
        v = port_mcl_colscale(cp, port_mcl_inflate(v, inflation))
        it += 1
    return canonical_csc(cp, ri, v), it, float(chaos)


def port_num_threads() -> int:
    return _port().gbc_o_num_threads()


# ------------------------------------------------------------------- helpers
def tuples_to_csc(rows, cols, vals, ncol):
    """Canonicalise a tuple list (any order) to CSC with rows sorted within
    each column (the comparison form for unsorted hash outputs)."""
    order = np.lexsort((rows, cols))
    rows, cols, vals = rows[order], cols[order], vals[order]
    cp = np.zeros(ncol + 1, np.int64)
    cp[1:] = np.cumsum(np.bincount(cols, minlength=ncol))
    return cp, rows, vals


def canonical_csc(cp, rows, vals):
    """Sort rows within each column (stable)."""
    ncol = len(cp) - 1
    cols = np.repeat(np.arange(ncol, dtype=np.int64), np.diff(cp))
    return tuples_to_csc(np.asarray(rows), cols, np.asarray(vals), ncol)
