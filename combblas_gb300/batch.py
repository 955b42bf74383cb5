"""Batched SpGEMM (many uneven products in one launch per pass, replayed as
a CUDA graph) and the autotuner that picks its column-class thresholds.

The autotuner times each candidate (s1, s2) -- the flop limits of the two
warp-kernel column classes; columns above s2 go to the block/tile kernel --
on the batch itself and caches the fastest per matrix-statistics class in a
JSON file, so later batches of the same class reuse the choice without
re-timing."""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

import numpy as np

from . import _lib as L
from .local import SR_CODES, VT_OF_DTYPE, Context, as_gbc_matrix, default_context

CANDIDATES = [(256, 4096), (256, 1024), (64, 2048), (256, 0), (0, 0)]


class Batch:
    """gbc_batch: products C_p = A_p * B_p built once, replayed by run()."""

    def __init__(self, As, Bs, sr: str = "plustimes", dtype=np.float64, s1: int = -1, s2: int = -1,
                 ctx: Context | None = None):
        self.ctx = ctx or default_context()
        assert len(As) == len(Bs) and len(As) > 0
        self.np = len(As)
        self.dtype = np.dtype(dtype)
        keep: list = []
        ga = (L.gbc_matrix * self.np)(*[as_gbc_matrix(A, keep, self.dtype) for A in As])
        gb = (L.gbc_matrix * self.np)(*[as_gbc_matrix(B, keep, self.dtype) for B in Bs])
        self.h = C.c_void_p()
        L.check(L.lib().gbc_batch_create(self.ctx.h, SR_CODES[sr], VT_OF_DTYPE[self.dtype], self.np, ga, gb,
                                         int(s1), int(s2), C.byref(self.h)))
        self._keep = keep  # host inputs were copied; device inputs are referenced

    def run(self) -> float:
        ms = C.c_double()
        L.check(L.lib().gbc_batch_run(self.h, C.byref(ms)))
        return ms.value

    def info(self, p: int):
        nzc, nnz, fl = C.c_int64(), C.c_int64(), C.c_int64()
        L.check(L.lib().gbc_batch_info(self.h, p, C.byref(nzc), C.byref(nnz), C.byref(fl)))
        return nzc.value, nnz.value, fl.value

    def flops(self) -> int:
        return sum(self.info(p)[2] for p in range(self.np))

    def result(self, p: int):
        nzc, nnz, _ = self.info(p)
        cp = np.empty(nzc + 1, np.int64)
        ir = np.empty(nnz, np.int64)
        num = np.empty(nnz, self.dtype)
        L.check(L.lib().gbc_batch_result(self.h, p, cp.ctypes.data, ir.ctypes.data if nnz else None,
                                         num.ctypes.data if nnz else None, L.GBC_HOST))
        return cp, ir, num

    def column_pointers(self, p: int) -> np.ndarray:
        """Product p's column pointers only (host copy)."""
        nzc, _, _ = self.info(p)
        cp = np.empty(nzc + 1, np.int64)
        L.check(L.lib().gbc_batch_result(self.h, p, cp.ctypes.data, None, None, L.GBC_HOST))
        return cp

    def result_device(self, p: int, nrow: int, ncol: int):
        """Product p as a DeviceMatrix (CSC over the stored columns of B_p,
        which must be a CSC matrix)."""
        import torch

        from .local import DeviceMatrix

        nzc, nnz, _ = self.info(p)
        tdt = {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32,
               np.dtype(np.int64): torch.int64, np.dtype(np.bool_): torch.bool}[self.dtype]
        cp = torch.empty(nzc + 1, dtype=torch.int64, device="cuda")
        ir = torch.empty(max(nnz, 1), dtype=torch.int64, device="cuda")
        num = torch.empty(max(nnz, 1), dtype=tdt, device="cuda")
        L.check(L.lib().gbc_batch_result(self.h, p, cp.data_ptr(), ir.data_ptr(), num.data_ptr(), L.GBC_DEVICE))
        return DeviceMatrix(nrow, ncol, cp, ir[:nnz], num[:nnz])

    def close(self):
        if self.h:
            L.lib().gbc_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def stats_class(As, Bs) -> str:
    """Statistics class of a batch: problem count, log2 of the largest row
    count and of the mean stored entries per column (coarse buckets)."""
    m = max(A.nrow for A in As)
    deg = np.mean([A.nnz / max(A.ncol, 1) for A in As])
    return f"p{len(As)}_m{int(np.log2(max(m, 1)))}_d{int(np.log2(1 + deg))}"


def default_cache() -> str:
    return os.environ.get("GBCOMB_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "gbcomb", "autotune.json"))


def autotune(As, Bs, sr: str = "plustimes", dtype=np.float64, cache: str | None = None, reps: int = 3,
             candidates=CANDIDATES, ctx: Context | None = None):
    """Return ((s1, s2), timings) for this batch's statistics class, timing the
    candidates on a cache miss and storing the winner."""
    cache = cache or default_cache()
    key = f"{sr}:{np.dtype(dtype).name}:{stats_class(As, Bs)}"
    data = json.load(open(cache)) if os.path.exists(cache) else {}
    if key in data:
        return tuple(data[key]["choice"]), data[key]["timings"]
    timings = {}
    for s1, s2 in candidates:
        b = Batch(As, Bs, sr, dtype, s1, s2, ctx)
        b.run()
        timings[f"{s1},{s2}"] = min(b.run() for _ in range(reps))
        b.close()
    best = min(timings, key=timings.get)
    choice = tuple(int(x) for x in best.split(","))
    data[key] = {"choice": list(choice), "timings": timings}
    os.makedirs(os.path.dirname(cache) or ".", exist_ok=True)
    with open(cache, "w") as f:
        json.dump(data, f, indent=1)
    return choice, timings
