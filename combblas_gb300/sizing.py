"""Learned output-column sizing (host side): features, training, persistence.

The model is trained on the GPU by the library's own kernels
(gbc_mlp_train) on the exact per-column counts of the symbolic pass
(estimateNNZ_Hash, mtSpGEMM.h:806) and then stands in for that pass in
GBC_SIZING_LEARNED products.  Columns whose count exceeds the predicted
capacity are recomputed exactly, so the product never changes.

Weights, normalisation and the capacity margin are saved as JSON, keyed by
the statistics class of the training matrices, so reruns reuse them.
"""
from __future__ import annotations

import ctypes as C
import sys
import json
import os

import numpy as np

from . import _lib as L
from .local import Context, as_gbc_matrix, default_context

NF = 6
FEATURE_NAMES = ["log2(1+nnz B col)", "log2(1+flop)", "log2(1+max A col len)", "log2(1+std A col len)",
                 "log2(1+row tiles touched)", "log2(1+rows)"]


def features(A, B, exact: bool = True, ctx: Context | None = None):
    """(features [nzc x 6] float32, flop [nzc], exact nnz [nzc] or None)."""
    ctx = ctx or default_context()
    keep: list = []
    ga = as_gbc_matrix(A, keep, np.float64)
    gb = as_gbc_matrix(B, keep, np.float64)
    ga.num = None
    gb.num = None
    nzc = gb.nzc
    feat = np.empty((max(nzc, 1), NF), np.float32)
    flop = np.empty(max(nzc, 1), np.int64)
    nnz = np.empty(max(nzc, 1), np.int64) if exact else None
    L.check(L.lib().gbc_spgemm_features(ctx.h, C.byref(ga), C.byref(gb), feat.ctypes.data, flop.ctypes.data,
                                        nnz.ctypes.data if exact else None, L.GBC_HOST))
    return feat[:nzc], flop[:nzc], (nnz[:nzc] if exact else None)


class SizingModel:
    """gbc_mlp: the sizing network on one context."""

    def __init__(self, ctx: Context | None = None, seed: int = 0):
        self.ctx = ctx or default_context()
        self.h = C.c_void_p()
        L.check(L.lib().gbc_mlp_create(self.ctx.h, C.c_uint64(seed), C.byref(self.h)))
        self.n_params = L.lib().gbc_mlp_num_params()
        self.info: dict = {}

    # -- training ---------------------------------------------------------
    def train(self, feat: np.ndarray, target: np.ndarray, steps: int = 400, lr: float = 3e-3) -> float:
        feat = np.ascontiguousarray(feat, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        loss = C.c_float()
        L.check(L.lib().gbc_mlp_train(self.ctx.h, self.h, feat.ctypes.data, target.ctypes.data, len(target), steps,
                                      lr, C.byref(loss), L.GBC_HOST))
        return loss.value

    def gradient(self, feat, target):
        feat = np.ascontiguousarray(feat, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        g = np.empty(self.n_params, np.float32)  # network params + loss occupy the first slots
        L.check(L.lib().gbc_mlp_gradient(self.ctx.h, self.h, feat.ctypes.data, target.ctypes.data, len(target),
                                         g.ctypes.data, L.GBC_HOST))
        return g

    def predict(self, feat: np.ndarray) -> np.ndarray:
        feat = np.ascontiguousarray(feat, np.float32)
        out = np.empty(len(feat), np.float32)
        L.check(L.lib().gbc_mlp_predict(self.ctx.h, self.h, feat.ctypes.data, len(feat), out.ctypes.data,
                                        L.GBC_HOST))
        return out

    def fit(self, feat, nnz, steps: int = 400, lr: float = 3e-3, quantile: float = 0.995) -> dict:
        """Train on exact counts and set the capacity margin so that about
        (1 - quantile) of the training columns would overflow."""
        nz = np.asarray(nnz) > 0
        target = np.log2(1.0 + np.asarray(nnz, np.float64)).astype(np.float32)
        loss = self.train(feat[nz], target[nz], steps, lr)
        resid = target[nz] - self.predict(feat[nz])
        margin = float(max(0.05, np.quantile(resid, quantile))) if nz.any() else 1.0
        self.set_margin(margin)
        self.info = {"loss": loss, "resid_std": float(resid.std()) if nz.any() else 0.0, "margin": margin,
                     "samples": int(nz.sum())}
        return self.info

    # -- parameters ------------------------------------------------------
    def get(self):
        p = np.empty(self.n_params, np.float32)
        m = C.c_float()
        L.check(L.lib().gbc_mlp_get(self.h, p.ctypes.data, C.byref(m)))
        return p, m.value

    def set(self, params: np.ndarray, margin: float):
        params = np.ascontiguousarray(params, np.float32)
        L.check(L.lib().gbc_mlp_set(self.h, params.ctypes.data, float(margin)))

    def set_margin(self, margin: float):
        p, _ = self.get()
        L.check(L.lib().gbc_mlp_set(self.h, None, float(margin)))

    def use(self):
        """Make this the model of GBC_SIZING_LEARNED on its context."""
        L.check(L.lib().gbc_context_set_mlp(self.ctx.h, self.h))

    def save(self, path: str, key: str = "default"):
        p, m = self.get()
        data = json.load(open(path)) if os.path.exists(path) else {}
        data[key] = {"params": [float(x) for x in p], "margin": m, "info": self.info}
        with open(path, "w") as f:
            json.dump(data, f)

    def load(self, path: str, key: str = "default") -> bool:
        if not os.path.exists(path):
            return False
        data = json.load(open(path))
        if key not in data:
            return False
        self.set(np.array(data[key]["params"], np.float32), data[key]["margin"])
        self.info = data[key].get("info", {})
        return True

    def close(self):
        if self.h:
            L.lib().gbc_context_set_mlp(self.ctx.h, None)
            L.lib().gbc_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def stats_class(A) -> str:
    """Coarse statistics class of a matrix (log2 of rows, of average degree)."""
    deg = A.nnz / max(A.ncol, 1)
    return f"m{int(np.log2(max(A.nrow, 1)))}_d{int(np.log2(1 + deg))}"
