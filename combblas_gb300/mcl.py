"""MCL on the GPU: the expansion step C = A*A over PlusTimes fp32 with the
prune/select/recovery of MCLPruneRecoverySelect (ParFriends.h:185-354), as
MemEfficientSpGEMM(..., phases=1, ...) runs it for Applications/MCL.cpp:573;
the vector steps MakeColStochastic, Chaos and Inflate (MCL.cpp:389-449); and
the whole HipMCL iteration loop (MCL.cpp:526-626) with the matrix kept on
the device."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .local import Context, SpResult, default_context

EPS = 0.0001  # the loop runs while chaos > EPS (MCL.cpp:55)


def MCLPruneRecoverySelect(Cres: SpResult, hardThreshold: float, selectNum: int, recoverNum: int = 0,
                           recoverPct: float = 0.0, ctx: Context | None = None):
    """Prune/select/recover a device fp32 product; returns a new SpResult.
    recoverNum == 0 disables recovery, as in the reference."""
    ctx = ctx or default_context()
    out = C.c_void_p()
    L.check(L.lib().gbc_mcl_prune_select_recover_f32(ctx.h, Cres.h, float(hardThreshold), int(selectNum),
                                                     int(recoverNum), float(recoverPct), C.byref(out)))
    return SpResult(out)


def _sizing(sizing: str) -> int:
    if sizing not in ("exact", "learned"):
        raise ValueError("sizing must be 'exact' or 'learned'")
    return L.SIZING_LEARNED if sizing == "learned" else L.SIZING_EXACT


def mcl_expand(A, hardThreshold: float = 1e-4, selectNum: int = 100, sizing: str = "exact", recoverNum: int = 0,
               recoverPct: float = 0.9, ctx: Context | None = None):
    """One expansion step: (A*A) pruned, selected and recovered, in one
    library call (gbc_mcl_expand_recover_f32).  Learned sizing feeds the
    select the capacity-slotted product directly.  Returns (result, SpGEMM
    statistics)."""
    from .local import as_gbc_matrix

    ctx = ctx or default_context()
    keep: list = []
    ga = as_gbc_matrix(A, keep, np.float32)
    out = C.c_void_p()
    st = L.gbc_spgemm_stats()
    L.check(L.lib().gbc_mcl_expand_recover_f32(ctx.h, C.byref(ga), float(hardThreshold), int(selectNum),
                                               int(recoverNum), float(recoverPct), _sizing(sizing), C.byref(out),
                                               C.byref(st)))
    return SpResult(out), st


def MakeColStochastic(R: SpResult, ctx: Context | None = None) -> SpResult:
    """Scale every column of a device fp32 result by 1 / (its sum), in place."""
    ctx = ctx or default_context()
    L.check(L.lib().gbc_mcl_make_col_stochastic_f32(ctx.h, R.h))
    return R


def Inflate(R: SpResult, power: float, ctx: Context | None = None) -> SpResult:
    """Raise every value of a device fp32 result to `power`, in place."""
    ctx = ctx or default_context()
    L.check(L.lib().gbc_mcl_inflate_f32(ctx.h, R.h, float(power)))
    return R


def Chaos(R: SpResult, ctx: Context | None = None) -> float:
    """max over columns of (column max - sum of squares) * nnz(column)."""
    ctx = ctx or default_context()
    c = C.c_float()
    L.check(L.lib().gbc_mcl_chaos_f32(ctx.h, R.h, C.byref(c)))
    return c.value


def HipMCL(A, inflation: float = 2.0, prunelimit: float = 1e-4, select: int = 1100, recover_num: int = 1400,
           recover_pct: float = 0.9, sizing: str = "exact", max_iter: int = 0, ctx: Context | None = None):
    """The HipMCL loop from the loop-adjusted matrix on, in one library call
    (gbc_mcl_iterate_f32); defaults are the application's (MCL.cpp:143-150).
    Returns (converged SpResult, iterations, last chaos)."""
    from .local import as_gbc_matrix

    ctx = ctx or default_context()
    keep: list = []
    ga = as_gbc_matrix(A, keep, np.float32)
    out = C.c_void_p()
    it = C.c_int64()
    chaos = C.c_float()
    L.check(L.lib().gbc_mcl_iterate_f32(ctx.h, C.byref(ga), float(inflation), float(prunelimit), int(select),
                                        int(recover_num), float(recover_pct), _sizing(sizing), int(max_iter),
                                        C.byref(out), C.byref(it), C.byref(chaos)))
    return SpResult(out), it.value, chaos.value
