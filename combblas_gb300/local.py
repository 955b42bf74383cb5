"""Host-side mirror of the reference's node-local kernel interface.

Names and argument meaning follow the reference calls the C ABI replaces:

* ``LocalHybridSpGEMM(A, B, clearA, clearB)`` -- mtSpGEMM.h:213-217 (and the
  CSC overload mtSpGEMM.h:1148-1152)
* ``LocalSpGEMM(A, B, clearA, clearB)`` -- mtSpGEMM.h:74-78 (heap variant,
  same product)
* ``LocalSpGEMMHash(A, B, clearA, clearB, sort)`` -- mtSpGEMM.h:463-467
* ``estimateFLOP(A, B)`` -- mtSpGEMM.h:1057; ``estimateNNZ_Hash(A, B)`` --
  mtSpGEMM.h:806
* ``MultiwayMerge(lists, mdim, ndim)`` -- MultiwayMerge.h:428-708 (the sum of
  several stages' products, equal entries combined in list order)
* ``dcsc_gespmv(A, x, y)`` / ``SpMVPlan`` -- Friends.h:63-175 (y (+)= A x with a
  dense vector)

The semiring is given by name (the reference's template argument ``SR``):
``"plustimes"`` (PlusTimesSRing), ``"minplus"`` (MinPlusSRing),
``"select2ndmin"`` (Select2ndMinSR), ``"bool"`` (PlusTimesSRing<bool,bool>).
``clearA``/``clearB`` are accepted for signature parity; Python owns its
arrays, so nothing is deleted.

Every call goes through libgbcomb.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import sys
from contextlib import contextmanager
from dataclasses import dataclass

import numpy as np

from . import _lib as L

SR_CODES = {"plustimes": L.SR_PLUSTIMES, "minplus": L.SR_MINPLUS, "select2ndmin": L.SR_SELECT2NDMIN,
            "bool": L.SR_BOOL}
VT_OF_DTYPE = {np.dtype(np.float64): L.VT_F64, np.dtype(np.float32): L.VT_F32, np.dtype(np.int64): L.VT_I64,
               np.dtype(np.bool_): L.VT_BOOL}
DTYPE_OF_VT = {v: k for k, v in VT_OF_DTYPE.items()}


class Context:
    """A device, a stream and the library's memory pool (gbc_context)."""

    def __init__(self, device: int = 0):
        self.h = C.c_void_p()
        L.check(L.lib().gbc_context_create(C.byref(self.h), device))
        self.device = device

    def synchronize(self):
        L.check(L.lib().gbc_context_synchronize(self.h))

    def set_stream(self, stream_handle: int | None):
        L.check(L.lib().gbc_context_set_stream(self.h, C.c_void_p(stream_handle or 0)))

    fold = "exact"

    def set_fold(self, fold: str):
        """How PlusTimes fp64 products are summed (gbc_context_set_fold):
        "exact" (default) -- the exact sum of the rounded products, rounded
        once; "ordered" -- the reference's hash-path left fold in B-entry
        order, bit for bit."""
        code = {"exact": L.FOLD_EXACT, "ordered": L.FOLD_ORDERED}[fold]
        L.check(L.lib().gbc_context_set_fold(self.h, code))
        self.fold = fold

    @contextmanager
    def folding(self, fold: str | None):
        """Temporarily use `fold` (None: leave the context as it is)."""
        if fold is None or fold == self.fold:
            yield self
            return
        old = self.fold
        self.set_fold(fold)
        try:
            yield self
        finally:
            self.set_fold(old)

    def close(self):
        if self.h:
            L.lib().gbc_context_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        # at interpreter exit objects are finalised in no particular order;
        # the process teardown releases the device memory
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


_default: dict[int, Context] = {}


def default_context(device: int = 0) -> Context:
    if device not in _default:
        _default[device] = Context(device)
    return _default[device]


@dataclass
class DCSC:
    """Host DCSC arrays as the reference's Dcsc holds them (dcsc.h:125-131)."""

    nrow: int
    ncol: int
    cp: np.ndarray
    jc: np.ndarray
    ir: np.ndarray
    numx: np.ndarray | None

    @staticmethod
    def from_csc(M) -> "DCSC":
        cnt = np.diff(M.colptr)
        jc = np.nonzero(cnt)[0].astype(np.int64)
        cp = np.concatenate([[0], np.cumsum(cnt[jc])]).astype(np.int64)
        return DCSC(M.nrow, M.ncol, cp, jc, M.rowidx, M.values)

    @property
    def nnz(self) -> int:
        return int(self.cp[-1])

    @property
    def nzc(self) -> int:
        return len(self.jc)


class DeviceMatrix:
    """Matrix arrays already resident on the device (torch tensors are used
    only as device buffers)."""

    def __init__(self, nrow, ncol, cp, ir, num=None, jc=None):
        self.nrow, self.ncol = int(nrow), int(ncol)
        self.cp, self.ir, self.num, self.jc = cp, ir, num, jc

    @staticmethod
    def from_host(M, device: str = "cuda", dtype=None) -> "DeviceMatrix":
        import torch

        if isinstance(M, DCSC):
            cp, jc, ir, v = M.cp, M.jc, M.ir, M.numx
        else:
            cp, jc, ir, v = M.colptr, None, M.rowidx, M.values
        if dtype is not None and v is not None:
            v = v.astype(dtype)
        t = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a)).to(device)
        return DeviceMatrix(M.nrow, M.ncol, t(cp), t(ir), t(v), t(jc))

    @property
    def nnz(self) -> int:
        return int(self.ir.numel())

    @property
    def nzc(self) -> int:
        return int(self.cp.numel()) - 1

    @property
    def dtype(self):
        if self.num is None:
            return None
        import torch

        return {torch.float64: np.dtype(np.float64), torch.float32: np.dtype(np.float32),
                torch.int64: np.dtype(np.int64), torch.bool: np.dtype(np.bool_)}[self.num.dtype]


def as_gbc_matrix(M, keep: list, dtype=None) -> L.gbc_matrix:
    """Describe a host CSC/DCSC or a DeviceMatrix as a gbc_matrix.  Arrays
    created here are appended to ``keep`` so they outlive the call."""
    g = L.gbc_matrix()
    if isinstance(M, DeviceMatrix):
        g.nrow, g.ncol = M.nrow, M.ncol
        g.nzc, g.nnz = M.nzc, M.nnz
        g.cp = M.cp.data_ptr()
        g.jc = M.jc.data_ptr() if M.jc is not None else None
        g.ir = M.ir.data_ptr() if M.nnz else None
        g.num = M.num.data_ptr() if (M.num is not None and M.nnz) else None
        g.where = L.GBC_DEVICE
        return g
    if isinstance(M, DCSC):
        cp, jc, ir, v = M.cp, M.jc, M.ir, M.numx
    else:
        cp, jc, ir, v = M.colptr, None, M.rowidx, M.values
    cp = np.ascontiguousarray(cp, np.int64)
    ir = np.ascontiguousarray(ir, np.int64)
    keep += [cp, ir]
    g.nrow, g.ncol = M.nrow, M.ncol
    g.nzc = len(cp) - 1
    g.nnz = int(cp[-1]) if len(cp) else 0
    g.cp = cp.ctypes.data
    g.ir = ir.ctypes.data if len(ir) else None
    if jc is not None:
        jc = np.ascontiguousarray(jc, np.int64)
        keep.append(jc)
        g.jc = jc.ctypes.data if len(jc) else None
        if not len(jc):
            g.jc = None
            g.nzc = 0 if g.ncol else 0
    if v is not None:
        v = np.ascontiguousarray(v, dtype) if dtype is not None else np.ascontiguousarray(v)
        keep.append(v)
        g.num = v.ctypes.data if len(v) else None
    g.where = L.GBC_HOST
    return g


class SpResult:
    """Device-resident product (gbc_result).  ``cp/jc`` describe the stored
    output columns; ``tuples()`` gives the SpTuples view (row, col, val)."""

    def __init__(self, handle: C.c_void_p, stats: L.gbc_spgemm_stats | None = None):
        self.h = handle
        self.stats = stats
        nrow, ncol, nzc, nnz = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        vt = C.c_int()
        L.check(L.lib().gbc_result_info(self.h, C.byref(nrow), C.byref(ncol), C.byref(nzc), C.byref(nnz),
                                         C.byref(vt)))
        self.nrow, self.ncol, self.nzc, self.nnz, self.vt = nrow.value, ncol.value, nzc.value, nnz.value, vt.value

    @property
    def dtype(self):
        return DTYPE_OF_VT[self.vt]

    def to_host(self):
        cp = np.empty(self.nzc + 1, np.int64)
        jc = np.empty(self.nzc, np.int64)
        ir = np.empty(self.nnz, np.int64)
        num = np.empty(self.nnz, self.dtype)
        L.check(L.lib().gbc_result_copy(self.h, cp.ctypes.data, jc.ctypes.data if self.nzc else None,
                                        ir.ctypes.data if self.nnz else None,
                                        num.ctypes.data if self.nnz else None, L.GBC_HOST))
        return cp, jc, ir, num

    def copy_to(self, cp, jc, ir, num, where=L.GBC_HOST):
        """Copy into caller buffers (raw addresses), host or device."""
        L.check(L.lib().gbc_result_copy(self.h, cp, jc, ir, num, where))

    def to_csc(self):
        """Dense-column CSC over all ncol columns (host arrays)."""
        cp, jc, ir, num = self.to_host()
        full = np.zeros(self.ncol + 1, np.int64)
        cnt = np.zeros(self.ncol, np.int64)
        cnt[jc] = np.diff(cp)
        full[1:] = np.cumsum(cnt)
        return full, ir, num

    def tuples(self):
        cp, jc, ir, num = self.to_host()
        cols = np.repeat(jc, np.diff(cp))
        return ir, cols, num

    def device_ptrs(self):
        p = [C.c_void_p() for _ in range(4)]
        L.check(L.lib().gbc_result_device_ptrs(self.h, *[C.byref(x) for x in p]))
        return [x.value for x in p]

    def free(self):
        if self.h:
            L.lib().gbc_result_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.free()
        except Exception:
            pass


def _value_dtype(A, B, sr: str):
    if sr == "bool":
        return np.dtype(np.bool_)
    for M in (A, B):
        d = M.dtype if isinstance(M, DeviceMatrix) else (
            None if (M.numx if isinstance(M, DCSC) else M.values) is None else
            (M.numx if isinstance(M, DCSC) else M.values).dtype)
        if d is not None:
            return np.dtype(d)
    return np.dtype(np.int64) if sr == "select2ndmin" else np.dtype(np.float64)


def spgemm(A, B, sr: str = "plustimes", sizing: str = "exact", sorted: bool = True, keep_empty: bool = True,
           ctx: Context | None = None, dtype=None, tile_rows: int = 0, tiny_limit: int = -1,
           small_limit: int = -1, fold: str | None = None) -> SpResult:
    """C = A * B over ``sr`` on the GPU.  tile_rows / tiny_limit /
    small_limit are tuning knobs (see gbc_spgemm_opts); results do not
    depend on them.  ``fold`` ("exact" / "ordered", None: the context's)
    selects how PlusTimes fp64 products are summed (Context.set_fold)."""
    ctx = ctx or default_context()
    dt = np.dtype(dtype) if dtype is not None else _value_dtype(A, B, sr)
    vt = VT_OF_DTYPE[dt]
    keep: list = []
    ga = as_gbc_matrix(A, keep, dt)
    gb = as_gbc_matrix(B, keep, dt)
    opts = L.gbc_spgemm_opts(L.SIZING_LEARNED if sizing == "learned" else L.SIZING_EXACT, int(bool(sorted)),
                             int(bool(keep_empty)), int(tile_rows), int(tiny_limit), int(small_limit))
    out = C.c_void_p()
    st = L.gbc_spgemm_stats()
    with ctx.folding(fold):
        L.check(L.lib().gbc_spgemm(ctx.h, SR_CODES[sr], vt, C.byref(ga), C.byref(gb), C.byref(opts), C.byref(out),
                                   C.byref(st)))
    return SpResult(out, st)


def spgemm_phased(A, B, sr: str = "plustimes", max_phase_nnz: int = 1 << 31, ctx: Context | None = None,
                  dtype=None, sizing: str = "exact", fold: str | None = None) -> L.gbc_phased_stats:
    """C = A * B in column phases of at most ``max_phase_nnz`` output entries;
    returns the statistics and checksums (the product is not kept).
    ``sizing="learned"`` sizes the phases with the context's sizing model
    (columns that overflow their predicted capacity are recomputed exactly)."""
    ctx = ctx or default_context()
    dt = np.dtype(dtype) if dtype is not None else _value_dtype(A, B, sr)
    keep: list = []
    ga = as_gbc_matrix(A, keep, dt)
    gb = as_gbc_matrix(B, keep, dt)
    st = L.gbc_phased_stats()
    with ctx.folding(fold):
        L.check(L.lib().gbc_spgemm_phased(ctx.h, SR_CODES[sr], VT_OF_DTYPE[dt], C.byref(ga), C.byref(gb),
                                          int(max_phase_nnz),
                                          L.SIZING_LEARNED if sizing == "learned" else L.SIZING_EXACT, C.byref(st)))
    return st


class SpMVPlan:
    """A, prepared for y <- y (+) A x (gbc_spmv_plan): dcsc_gespmv
    (Friends.h:63-175) with A's rows held row-major on the device."""

    def __init__(self, A, dtype=np.float64, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.dtype = np.dtype(dtype)
        keep: list = []
        g = as_gbc_matrix(A, keep, self.dtype)
        self.h = C.c_void_p()
        L.check(L.lib().gbc_spmv_plan_create(self.ctx.h, VT_OF_DTYPE[self.dtype], C.byref(g), C.byref(self.h)))
        self.nrow, self.ncol = int(A.nrow), int(A.ncol)

    def multiply(self, x, y, sr: str = "plustimes"):
        """y (+)= A x; numpy arrays (updated in place and returned) or device
        addresses (ints)."""
        if isinstance(x, int):
            L.check(L.lib().gbc_spmv(self.ctx.h, self.h, SR_CODES[sr], C.c_void_p(x), C.c_void_p(y), L.GBC_DEVICE))
            return y
        x = np.ascontiguousarray(x, self.dtype)
        assert y.dtype == self.dtype and y.flags.c_contiguous
        L.check(L.lib().gbc_spmv(self.ctx.h, self.h, SR_CODES[sr], x.ctypes.data, y.ctypes.data, L.GBC_HOST))
        return y

    def close(self):
        if self.h:
            L.lib().gbc_spmv_plan_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def dcsc_gespmv(A, x, y, sr: str = "plustimes", dtype=None):
    """y (+)= A x, the reference's dcsc_gespmv (one-shot plan)."""
    dt = np.dtype(dtype) if dtype is not None else np.asarray(y).dtype
    plan = SpMVPlan(A, dt)
    try:
        return plan.multiply(x, y, sr)
    finally:
        plan.close()


def MultiwayMerge(lists, mdim: int, ndim: int, sr: str = "plustimes", dtype=None,
                  ctx: Context | None = None) -> SpResult:
    """Sum of matrices of one shape with duplicates combined by the
    semiring's add in list order (MultiwayMerge.h:428-708)."""
    ctx = ctx or default_context()
    if lists:
        dt = np.dtype(dtype) if dtype is not None else _value_dtype(lists[0], lists[0], sr)
    else:
        dt = np.dtype(dtype or np.float64)
    keep: list = []
    arr = (L.gbc_matrix * max(len(lists), 1))(*[as_gbc_matrix(M, keep, dt) for M in lists])
    out = C.c_void_p()
    st = L.gbc_spgemm_stats()
    L.check(L.lib().gbc_multiway_merge(ctx.h, SR_CODES[sr], VT_OF_DTYPE[dt], len(lists), arr, int(mdim), int(ndim),
                                       C.byref(out), C.byref(st)))
    return SpResult(out, st)


def LocalHybridSpGEMM(A, B, clearA: bool = False, clearB: bool = False, sr: str = "plustimes", **kw) -> SpResult:
    return spgemm(A, B, sr=sr, **kw)


def LocalSpGEMM(A, B, clearA: bool = False, clearB: bool = False, sr: str = "plustimes", **kw) -> SpResult:
    return spgemm(A, B, sr=sr, **kw)


def LocalSpGEMMHash(A, B, clearA: bool = False, clearB: bool = False, sort: bool = True, sr: str = "plustimes",
                    **kw) -> SpResult:
    return spgemm(A, B, sr=sr, sorted=sort, **kw)


def _colstats(A, B, ctx=None):
    ctx = ctx or default_context()
    keep: list = []
    ga = as_gbc_matrix(A, keep, np.float64)
    gb = as_gbc_matrix(B, keep, np.float64)
    ga.num = None
    gb.num = None
    flop = np.empty(max(gb.nzc, 1), np.int64)
    nnz = np.empty(max(gb.nzc, 1), np.int64)
    L.check(L.lib().gbc_spgemm_colstats(ctx.h, C.byref(ga), C.byref(gb), flop.ctypes.data, nnz.ctypes.data,
                                        L.GBC_HOST))
    return flop[:gb.nzc], nnz[:gb.nzc]


def estimateFLOP(A, B, ctx=None) -> np.ndarray:
    """Per stored column of B: the number of multiplications."""
    return _colstats(A, B, ctx)[0]


def estimateNNZ_Hash(A, B, ctx=None) -> np.ndarray:
    """Per stored column of B: the exact nnz of that column of A*B."""
    return _colstats(A, B, ctx)[1]
