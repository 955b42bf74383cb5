"""SpMSpV over SelectMin and the BFS built on it -- host mirror of
``SpMXSpV_Bucket`` (SpImpl.cpp:389) and the BFS_CSC level loop of
Applications/SpMSpV-IPDPS2017/SpMSpVBench.cpp:128-156 -- plus the
multi-source BFS of the Select2ndMin SpGEMM loop in
Applications/Ordering/MD.cpp:211-217.  GPU only."""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np

from . import _lib as L
from .local import Context, DeviceMatrix, as_gbc_matrix, default_context


class Graph:
    """Square pattern matrix prepared once on the device (gbc_graph)."""

    def __init__(self, A, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        keep: list = []
        g = as_gbc_matrix(A, keep, None)
        g.num = None
        self.h = C.c_void_p()
        L.check(L.lib().gbc_graph_create(self.ctx.h, C.byref(g), C.byref(self.h)))
        self.n = int(A.ncol)
        self.colptr = A.colptr if not isinstance(A, DeviceMatrix) else None

    def set_policy(self, policy: str):
        """"auto" (per-level direction), "topdown" or "bottomup"."""
        L.check(L.lib().gbc_graph_set_policy(self.h, {"auto": 0, "topdown": 1, "bottomup": 2}[policy]))

    def close(self):
        if self.h:
            L.lib().gbc_graph_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def SpMXSpV(graph: Graph, indx: np.ndarray, numx: np.ndarray):
    """y = A x over SelectMin: returns (indy int32 sorted, numy int64)."""
    indx = np.ascontiguousarray(indx, np.int32)
    numx = np.ascontiguousarray(numx, np.int64)
    indy = np.empty(graph.n, np.int32)
    numy = np.empty(graph.n, np.int64)
    ny = C.c_int32()
    L.check(L.lib().gbc_spmspv_select2ndmin_i64(graph.ctx.h, graph.h, indx.ctypes.data, numx.ctypes.data, len(indx),
                                                indy.ctypes.data, numy.ctypes.data, C.byref(ny), L.GBC_HOST))
    return indy[:ny.value].copy(), numy[:ny.value].copy()


_SX = {"select2ndmin": L.SR_SELECT2NDMIN, "selectmin": L.SR_SELECT2NDMIN, "select2nd": L.SR_SELECT2ND,
       "selectmax": L.SR_SELECTMAX, "plustimes": L.SR_PLUSTIMES}
_VT = {np.dtype(np.float64): L.VT_F64, np.dtype(np.float32): L.VT_F32, np.dtype(np.int64): L.VT_I64,
       np.dtype(np.bool_): L.VT_BOOL}


class SpMSpVPlan:
    """Any m x n matrix held on the device for repeated sparse-vector
    multiplies over the reference's SpMXSpV semirings (gbc_spmspv_plan):
    "select2ndmin" / "selectmin", "select2nd" (the value of the largest
    hitting column, TopDownBFS's boolean Select2ndSRing), "selectmax" and
    "plustimes" (ascending-column left fold, as SpMXSpV_Bucket).  dtype is
    the value type of A and, for plustimes, of x and y; None keeps only the
    pattern (the select semirings)."""

    def __init__(self, A, dtype=None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        keep: list = []
        self.dtype = np.dtype(dtype) if dtype is not None else np.dtype(np.bool_)
        g = as_gbc_matrix(A, keep, None if dtype is None else self.dtype.type)
        if dtype is None:
            g.num = None
        self.h = C.c_void_p()
        L.check(L.lib().gbc_spmspv_plan_create(self.ctx.h, _VT[self.dtype], C.byref(g), C.byref(self.h)))
        self.m, self.n = int(A.nrow), int(A.ncol)

    def multiply(self, indx, numx, semiring: str = "select2ndmin"):
        """y = A x: returns (indy int32 ascending, numy)."""
        sr = _SX[semiring]
        dt = self.dtype if sr == L.SR_PLUSTIMES else np.dtype(np.int64)
        indx = np.ascontiguousarray(indx, np.int32)
        numx = np.ascontiguousarray(numx, dt)
        indy = np.empty(max(self.m, 1), np.int32)
        numy = np.empty(max(self.m, 1), dt)
        ny = C.c_int32()
        L.check(L.lib().gbc_spmspv(self.ctx.h, self.h, sr, indx.ctypes.data, numx.ctypes.data, len(indx),
                                   indy.ctypes.data, numy.ctypes.data, C.byref(ny), L.GBC_HOST))
        return indy[:ny.value].copy(), numy[:ny.value].copy()

    def close(self):
        if self.h:
            L.lib().gbc_spmspv_plan_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def bfs(A_or_graph, source: int, ctx: Context | None = None):
    """BFS from ``source``: (parents int64[n], levels int64[n], stats)."""
    g = A_or_graph if isinstance(A_or_graph, Graph) else Graph(A_or_graph, ctx)
    parents = np.empty(g.n, np.int64)
    levels = np.empty(g.n, np.int64)
    st = L.gbc_bfs_stats()
    L.check(L.lib().gbc_bfs(g.ctx.h, g.h, int(source), parents.ctypes.data, levels.ctypes.data, C.byref(st),
                            L.GBC_HOST))
    return parents, levels, st


def bfs_device(graph: Graph, source: int, parents_ptr: int, levels_ptr: int):
    """BFS writing into caller device buffers (int64[n] each); the level
    loop then runs as a captured CUDA graph."""
    st = L.gbc_bfs_stats()
    L.check(L.lib().gbc_bfs(graph.ctx.h, graph.h, int(source), C.c_void_p(parents_ptr), C.c_void_p(levels_ptr),
                            C.byref(st), L.GBC_DEVICE))
    return st


def msbfs(graph: Graph, roots, parents_ptr: int | None = None):
    """BFS from every root at once (F_{l+1} = A * F_l masked by visited,
    Select2ndMin, values = row ids).  Returns (parents int64[len(roots), n]
    or None when written to the device buffer at ``parents_ptr``, stats)."""
    roots = np.ascontiguousarray(roots, np.int64)
    st = L.gbc_msbfs_stats()
    if parents_ptr is None:
        parents = np.empty((len(roots), graph.n), np.int64)
        L.check(L.lib().gbc_msbfs(graph.ctx.h, graph.h, roots.ctypes.data, len(roots), parents.ctypes.data,
                                  L.GBC_HOST, C.byref(st)))
        return parents, st
    L.check(L.lib().gbc_msbfs(graph.ctx.h, graph.h, roots.ctypes.data, len(roots), C.c_void_p(parents_ptr),
                              L.GBC_DEVICE, C.byref(st)))
    return None, st
