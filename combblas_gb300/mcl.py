"""MCL expansion step on the GPU: C = A*A over PlusTimes fp32, then the
prune/select of MCLPruneRecoverySelect (ParFriends.h:185-354) with
recoverNum = 0, as MemEfficientSpGEMM(..., phases=1, ...) runs it for
Applications/MCL.cpp:573."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .local import Context, SpResult, default_context, spgemm


def MCLPruneRecoverySelect(Cres: SpResult, hardThreshold: float, selectNum: int, ctx: Context | None = None):
    """Prune/select a device fp32 product; returns a new SpResult."""
    ctx = ctx or default_context()
    out = C.c_void_p()
    L.check(L.lib().gbc_mcl_prune_select_f32(ctx.h, Cres.h, float(hardThreshold), int(selectNum), C.byref(out)))
    return SpResult(out)


def mcl_expand(A, hardThreshold: float = 1e-4, selectNum: int = 100, sizing: str = "exact",
               ctx: Context | None = None):
    """One expansion step: (A*A) pruned and selected, in one library call
    (gbc_mcl_expand_f32).  Learned sizing feeds the select the capacity-
    slotted product directly.  Returns (result, SpGEMM statistics)."""
    from .local import as_gbc_matrix

    ctx = ctx or default_context()
    keep: list = []
    ga = as_gbc_matrix(A, keep, np.float32)
    out = C.c_void_p()
    st = L.gbc_spgemm_stats()
    L.check(L.lib().gbc_mcl_expand_f32(ctx.h, C.byref(ga), float(hardThreshold), int(selectNum),
                                       L.SIZING_LEARNED if sizing == "learned" else L.SIZING_EXACT, C.byref(out),
                                       C.byref(st)))
    return SpResult(out), st
