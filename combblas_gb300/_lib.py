"""ctypes binding of libgbcomb.so (the C ABI declared in include/gbcomb.h).

The library is loaded from the package directory only; if it is missing the
import fails loudly -- there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbcomb.so")

GBC_OK = 0
GBC_HOST = 0
GBC_DEVICE = 1

SR_PLUSTIMES = 0
SR_MINPLUS = 1
SR_SELECT2NDMIN = 2
SR_BOOL = 3
SR_SELECT2ND = 4
SR_SELECTMAX = 5

VT_F64 = 0
VT_F32 = 1
VT_I64 = 2
VT_BOOL = 3

SIZING_EXACT = 0
SIZING_LEARNED = 1

FOLD_EXACT = 0    # PlusTimes fp64: exact sum of the rounded products, rounded once
FOLD_ORDERED = 1  # PlusTimes fp64: left fold in B-entry order (the reference's hash path)


class GbcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbcomb error {code}: {msg}")
        self.code = code


class gbc_matrix(C.Structure):
    _fields_ = [
        ("nrow", C.c_int64), ("ncol", C.c_int64), ("nzc", C.c_int64), ("nnz", C.c_int64),
        ("cp", C.c_void_p), ("jc", C.c_void_p), ("ir", C.c_void_p), ("num", C.c_void_p),
        ("where", C.c_int),
    ]


class gbc_spgemm_opts(C.Structure):
    _fields_ = [("sizing", C.c_int), ("sorted", C.c_int), ("keep_empty", C.c_int), ("tile_rows", C.c_int),
                ("tiny_limit", C.c_int64), ("small_limit", C.c_int64)]


class gbc_spgemm_stats(C.Structure):
    _fields_ = [
        ("flops", C.c_int64), ("nnz", C.c_int64), ("overflow_cols", C.c_int64), ("alloc_entries", C.c_int64),
        ("ms_total", C.c_double), ("ms_symbolic", C.c_double), ("ms_numeric", C.c_double),
        ("tile_visits_dense", C.c_int64), ("tile_visits_range", C.c_int64),
    ]


class gbc_phased_stats(C.Structure):
    _fields_ = [
        ("flops", C.c_int64), ("nnz", C.c_int64), ("phases", C.c_int64), ("max_phase_nnz", C.c_int64),
        ("row_checksum", C.c_int64), ("val_checksum", C.c_double), ("content_hash", C.c_uint64),
        ("overflow_cols", C.c_int64), ("alloc_nnz", C.c_int64), ("ms_total", C.c_double),
        ("ms_sizing", C.c_double), ("ms_numeric", C.c_double), ("ms_rerun", C.c_double),
    ]


class gbc_bfs_stats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int64), ("reached", C.c_int64), ("edges", C.c_int64), ("ms", C.c_double),
        ("host_checks", C.c_int64),
    ]


class gbc_msbfs_stats(C.Structure):
    _fields_ = [
        ("levels", C.c_int64), ("reached", C.c_int64), ("edges", C.c_int64), ("ms", C.c_double),
        ("host_checks", C.c_int64),
    ]


_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "gbc_last_error": (C.c_char_p, []),
    "gbc_version": (C.c_int, []),
    "gbc_launch_count": (C.c_int64, []),
    "gbc_context_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "gbc_context_destroy": (C.c_int, [C.c_void_p]),
    "gbc_context_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gbc_context_set_fold": (C.c_int, [C.c_void_p, C.c_int]),
    "gbc_context_synchronize": (C.c_int, [C.c_void_p]),
    "gbc_result_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    "gbc_result_copy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "gbc_result_device_ptrs": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                         C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "gbc_result_free": (C.c_int, [C.c_void_p]),
    "gbc_spgemm": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(gbc_matrix), C.POINTER(gbc_matrix),
                             C.POINTER(gbc_spgemm_opts), C.POINTER(C.c_void_p), C.POINTER(gbc_spgemm_stats)]),
    "gbc_spgemm_phased": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(gbc_matrix), C.POINTER(gbc_matrix),
                                    C.c_int64, C.c_int, C.POINTER(gbc_phased_stats)]),
    "gbc_spgemm_colstats": (C.c_int, [C.c_void_p, C.POINTER(gbc_matrix), C.POINTER(gbc_matrix), C.c_void_p,
                                      C.c_void_p, C.c_int]),
}
for _n in ("plustimes_f64", "plustimes_f32", "plustimes_i64", "minplus_f64", "minplus_i64", "select2ndmin_i64"):
    _SIGS[f"gbc_spgemm_{_n}_i64"] = (C.c_int, [C.c_void_p, C.POINTER(gbc_matrix), C.POINTER(gbc_matrix),
                                               C.POINTER(gbc_spgemm_opts), C.POINTER(C.c_void_p),
                                               C.POINTER(gbc_spgemm_stats)])
_SIGS["gbc_spgemm_bool_i64"] = _SIGS["gbc_spgemm_plustimes_f64_i64"]
_SIGS.update({
    "gbc_batch_create": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(gbc_matrix),
                                   C.POINTER(gbc_matrix), C.c_int64, C.c_int64, C.POINTER(C.c_void_p)]),
    "gbc_batch_run": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "gbc_batch_info": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int64)]),
    "gbc_batch_result": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "gbc_batch_destroy": (C.c_int, [C.c_void_p]),
    "gbc_mlp_create": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "gbc_mlp_destroy": (C.c_int, [C.c_void_p]),
    "gbc_mlp_num_params": (C.c_int, []),
    "gbc_mlp_get": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_float)]),
    "gbc_mlp_set": (C.c_int, [C.c_void_p, C.c_void_p, C.c_float]),
    "gbc_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_float,
                                C.POINTER(C.c_float), C.c_int]),
    "gbc_mlp_gradient": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int]),
    "gbc_mlp_predict": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int]),
    "gbc_context_set_mlp": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gbc_spgemm_features": (C.c_int, [C.c_void_p, C.POINTER(gbc_matrix), C.POINTER(gbc_matrix), C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_int]),
    "gbc_mcl_expand_f32": (C.c_int, [C.c_void_p, C.POINTER(gbc_matrix), C.c_float, C.c_int64, C.c_int,
                                     C.POINTER(C.c_void_p), C.POINTER(gbc_spgemm_stats)]),
    "gbc_spmspv_plan_create": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(gbc_matrix), C.POINTER(C.c_void_p)]),
    "gbc_spmspv_plan_destroy": (C.c_int, [C.c_void_p]),
    "gbc_spmspv_plan_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int64)]),
    "gbc_spmspv": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                             C.c_void_p, C.POINTER(C.c_int32), C.c_int]),
    "gbc_mcl_prune_select_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_float, C.c_int64, C.POINTER(C.c_void_p)]),
    "gbc_mcl_prune_select_recover_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_float, C.c_int64, C.c_int64,
                                                   C.c_float, C.POINTER(C.c_void_p)]),
    "gbc_mcl_expand_recover_f32": (C.c_int, [C.c_void_p, C.POINTER(gbc_matrix), C.c_float, C.c_int64, C.c_int64,
                                             C.c_float, C.c_int, C.POINTER(C.c_void_p),
                                             C.POINTER(gbc_spgemm_stats)]),
    "gbc_mcl_make_col_stochastic_f32": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gbc_mcl_inflate_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double]),
    "gbc_mcl_chaos_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_float)]),
    "gbc_mcl_iterate_f32": (C.c_int, [C.c_void_p, C.POINTER(gbc_matrix), C.c_double, C.c_float, C.c_int64,
                                      C.c_int64, C.c_float, C.c_int, C.c_int64, C.POINTER(C.c_void_p),
                                      C.POINTER(C.c_int64), C.POINTER(C.c_float)]),
    "gbc_graph_create": (C.c_int, [C.c_void_p, C.POINTER(gbc_matrix), C.POINTER(C.c_void_p)]),
    "gbc_graph_destroy": (C.c_int, [C.c_void_p]),
    "gbc_graph_set_policy": (C.c_int, [C.c_void_p, C.c_int]),
    "gbc_spmspv_select2ndmin_i64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                              C.c_void_p, C.POINTER(C.c_int32), C.c_int]),
    "gbc_spmspv_select2ndmin_noalloc": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                                  C.POINTER(C.c_int32), C.c_void_p]),
    "gbc_bfs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(gbc_bfs_stats),
                          C.c_int]),
    "gbc_msbfs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int,
                            C.POINTER(gbc_msbfs_stats)]),
    "gbc_spmv_plan_create": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(gbc_matrix), C.POINTER(C.c_void_p)]),
    "gbc_spmv_plan_destroy": (C.c_int, [C.c_void_p]),
    "gbc_spmv": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "gbc_multiway_merge": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_int64,
                                     C.POINTER(C.c_void_p), C.POINTER(gbc_spgemm_stats)]),
})

# entry points added by later modules register here (see extend_signatures)
_EXTRA: dict = {}


def extend_signatures(sigs: dict) -> None:
    _EXTRA.update(sigs)
    if _lib is not None:
        _declare(_lib, sigs)


def _declare(lib, sigs):
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    """Load libgbcomb.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m combblas_gb300.build` "
                              "(the CUDA path has no CPU fallback)")
        l = C.CDLL(LIB_PATH)
        _declare(l, _SIGS)
        _declare(l, _EXTRA)
        _lib = l
    return _lib


def exported_symbols() -> list[str]:
    return sorted(set(_SIGS) | set(_EXTRA))


def check(rc: int) -> None:
    if rc != GBC_OK:
        msg = lib().gbc_last_error()
        raise GbcError(rc, msg.decode() if msg else "")
