"""ctypes binding of the C ABI in ``include/smolyax_gb300.h``.

The shared library is built in-tree (``smolyax_gb300/build.py``) and loaded
from ``smolyax_gb300/_lib``.  There is no fallback: if the library is missing
or no CUDA device is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libsmolyax_gb300.so")

SMX_OK = 0
SMX_ERR_ARG = -1
SMX_SERVE_BLOCKED = 0
SMX_SERVE_SPECTRAL = 1
SMX_MODE_NONZERO = 0
SMX_MODE_INDEXSET = 1
SMX_MODE_ADDITIVE = 2
SMX_MODE_PREORDER = 3
SMX_MAX_DEPTH = 64

_p = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_int = C.c_int
_dbl = C.c_double
_sz = C.c_size_t


class SmxPlan(C.Structure):
    """Mirror of ``struct smx_plan``."""

    _fields_ = [
        ("d_in", _i32),
        ("d_out", _i32),
        ("n_pairs", _i32),
        ("n_values", _i32),
        ("n_summands", _i32),
        ("max_n", _i32),
        ("n_entries", _i64),
        ("pair_dim", _p),
        ("pair_deg", _p),
        ("pair_voff", _p),
        ("node", _p),
        ("bweight", _p),
        ("sum_poff", _p),
        ("sum_pairs", _p),
        ("sum_eoff", _p),
        ("F64", _p),
        ("F32", _p),
        ("offset", _p),
        ("fp32", _p),
    ]


class SmxTree(C.Structure):
    """Mirror of ``struct smx_tree``."""

    _fields_ = [
        ("n", _i64),
        ("parent", _p),
        ("dim", _p),
        ("deg", _p),
        ("rem", _p),
        ("first_child", _p),
        ("n_child", _p),
    ]


class SmxSpectral(C.Structure):
    """Mirror of ``struct smx_spectral``."""

    _fields_ = [
        ("d_in", _i32),
        ("d_out", _i32),
        ("dstride", _i32),
        ("row", _i32),
        ("n_hb", _i32),
        ("n_vp", _i32),
        ("n_hot_dims", _i32),
        ("n_nodes", _i32),
        ("n_cold_groups", _i32),
        ("max_depth", _i32),
        ("n_cold_blocks", _i32),
        ("node_seg", _i32 * 5),
        ("cold_seg", _i32 * 5),
        ("block_seg", _i32 * 5),
        ("hot_dim", _p),
        ("hot_deg", _p),
        ("hot_soff", _p),
        ("node", _p),
        ("node_c", _p),
        ("cold", _p),
        ("cold_ab", _p),
        ("blk_dims", _p),
        ("blk_run", _p),
        ("blk_ab", _p),
        ("run", _p),
        ("coef", _p),
        ("fam_a", _p),
        ("fam_b", _p),
        ("fam", _p),
        ("c0", _p),
    ]


class SmxSpectral64(C.Structure):
    """Mirror of ``struct smx_spectral64``."""

    _fields_ = [
        ("d_in", _i32),
        ("d_out", _i32),
        ("dstride", _i32),
        ("row", _i32),
        ("n_hb", _i32),
        ("n_vp", _i32),
        ("n_hot_dims", _i32),
        ("n_nodes", _i32),
        ("n_cold_groups", _i32),
        ("max_depth", _i32),
        ("n_terms", _i32),
        ("node_seg", _i32 * 5),
        ("cold_seg", _i32 * 5),
        ("hot_dim", _p),
        ("hot_deg", _p),
        ("hot_soff", _p),
        ("node", _p),
        ("node_c", _p),
        ("cold", _p),
        ("cold_ab", _p),
        ("run", _p),
        ("terms", _p),
        ("coef", _p),
        ("fam_a", _p),
        ("fam_b", _p),
        ("fam", _p),
        ("c0", _p),
    ]


class SmxBlocked(C.Structure):
    """Mirror of ``struct smx_blocked``."""

    _fields_ = [
        ("d_in", _i32),
        ("n_hs", _i32),
        ("k_c", _i32),
        ("n_hot_dims", _i32),
        ("n_nodes", _i32),
        ("n_groups", _i32),
        ("n_items", _i32),
        ("c0", C.c_float),
        ("hot_dim", _p),
        ("hot_deg", _p),
        ("hot_soff", _p),
        ("node", _p),
        ("vc", _p),
        ("hot_ent", _p),
        ("grp", _p),
        ("grp_ab", _p),
        ("W", _p),
        ("warp_off", _p),
        ("items", _p),
        ("fa", _p),
        ("fb", _p),
        ("fam", _p),
        ("n_ent", _i32),
        ("n_w", _i32),
    ]


class SmxBlockedTc(C.Structure):
    """Mirror of ``struct smx_blocked_tc``."""

    _fields_ = [
        ("d_in", _i32),
        ("n_td", _i32),
        ("n_phi", _i32),
        ("n_phi_pad", _i32),
        ("n_rows", _i32),
        ("max_depth", _i32),
        ("n_agen", _i32),
        ("n_chunks", _i32),
        ("n_boxes", _i32),
        ("lin0", _i32),
        ("stages", _i32),
        ("td_col", _i32),
        ("td_bytes", _i32),
        ("c0", C.c_float),
        ("td", _p),
        ("tdab", _p),
        ("row", _p),
        ("chunk", _p),
        ("bimg", _p),
        ("box", _p),
        ("err", _p),
    ]


class SmxWork(C.Structure):
    """Mirror of ``struct smx_work``."""

    _fields_ = [("plan", _i32), ("reserved", _i32), ("x", _p), ("P", _i64), ("ldx", _i64), ("y", _p)]


# name -> (restype, argtypes); must list every function declared in the header.
SIGNATURES = {
    "smx_lambda_count": (_int, [_p, _int, _dbl, _int, _p, _p, _i64, _p, _p, _p]),
    "smx_lambda_expand": (_int, [_p, _int, _dbl, _int, _p, _p, _i64, _p, _i64, _p, _p, _p, _p, _p, _p]),
    "smx_zeta": (_int, [_p, _int, _p, _p, _i64, _p, _p, _p]),
    "smx_scan_workspace": (_sz, [_i64]),
    "smx_scan_i64": (_int, [_p, _p, _i64, _p, _sz, _p]),
    "smx_lambda_subtree_sizes": (_int, [_p, _p, _i64, _i64, _p, _p]),
    "smx_lambda_ranks": (_int, [_int, _p, _p, _p, _p, _p, _i64, _i64, _p, _p, _p]),
    "smx_bary_weights": (_int, [_int, _p, _p, _p, _p, _p]),
    "smx_plan_summands": (_int, [_i64, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    "smx_max_degree": (_int, [_i64, _p, _p, _p, _p]),
    "smx_assemble_F": (_int, [_p, _p, _p, _p, _p, _p, _p, _p]),
    "smx_basis_f64": (_int, [_p, _p, _i64, _i64, _p, _p, _p]),
    "smx_contract_f64": (_int, [_p, _p, _i64, _p, _p]),
    "smx_eval_workspace": (_sz, [_p, _i64, _int]),
    "smx_eval": (_int, [_p, _int, _p, _i64, _i64, _p, _p, _sz, _p]),
    "smx_jacobian_workspace": (_sz, [_p, _i64]),
    "smx_jacobian": (_int, [_p, _p, _i64, _i64, _p, _p, _sz, _p]),
    "smx_integral_workspace": (_sz, [_p]),
    "smx_integral": (_int, [_p, _p, _p, _p, _sz, _p]),
    "smx_spectral_pairs": (_int, [_int, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    "smx_spectral_coefficients": (_int, [_p, _p, _p, _p, _p, _p, _p, _i64, _p, _p, _p, _p, _p, _sz, _p]),
    "smx_spectral_coefficients_workspace": (_sz, [_p]),
    "smx_spectral_eval": (_int, [_p, _p, _i64, _i64, _p, _p]),
    "smx_spectral_eval64": (_int, [_p, _p, _i64, _i64, _p, _p]),
    "smx_blocked_smem": (_sz, [_p]),
    "smx_gemm_bf16x3": (_int, [_p, _p, _i64, _p, _p, _i64, _int, _int, _int, _p, _i64, _p, _int, _p, _p]),
    "smx_split_bf16": (_int, [_p, _i64, _i64, _i64, _p, _p, _i64, _p]),
    "smx_host_device_pointer": (_int, [_p, _p]),
    "smx_blocked_eval": (_int, [_p, _p, _i64, _i64, _p, _p, _sz, _p]),
    "smx_blocked_tc_eval": (_int, [_p, _p, _i64, _i64, _p, _p]),
    "smx_blocked_tc_supported": (_int, [_p, _p, _i64]),
    "smx_blocked_eval_workspace": (_sz, [_p, _i64]),
    "smx_blocked_eval_batch_workspace": (_sz, [_int, _int]),
    "smx_blocked_eval_batch": (_int, [_p, _int, _p, _int, _p, _sz, _p]),
    "smx_serve_create": (_int, [_int, _int, _int, _p, C.POINTER(_p)]),
    "smx_serve_submit": (_i64, [_p, _int, _p, _p, _i64, _i64, _p]),
    "smx_serve_flush": (_int, [_p]),
    "smx_serve_poll": (_int, [_p, _i64]),
    "smx_serve_destroy": (None, [_p]),
    "smx_eval_f64_noalloc": (_int, [_p, _p, _i64, _i64, _p, _p]),
    "smx_spectral_panel_workspace": (_sz, [_int, _i64]),
    "smx_spectral_panel_tf32": (_int, [_int, _p, _p, _p, _int, _p, _int, _p, _int, _p, _p, _p, _p, _i64, _i64, _p,
                                        _p, _i64, _p, _sz, _p]),
    "smx_spectral_panel_bf16": (_int, [_int, _p, _p, _p, _int, _p, _int, _p, _int, _p, _p, _p, _p, _i64, _i64, _p,
                                        _p, _i64, _p, _sz, _p]),
    "smx_spectral_eval_batch_workspace": (_sz, [_int, _int, _int]),
    "smx_spectral_eval_batch": (_int, [_p, _int, _p, _int, _p, _sz, _p]),
    "smx_gemm_tf32x3": (_int, [_p, _p, _i64, _p, _p, _i64, _int, _int, _int, _p, _i64, _p, _int, _p, _p]),
    "smx_gemm_tf32x3_timeout_selftest": (_int, [_p, _p, _i64, _p, _p, _i64, _int, _int, _int, _p, _i64, _p,
                                                 C.c_uint64, _p]),
    "smx_gemm_tf32x3_splitk_workspace": (_sz, [_int, _int, _int, _int]),
    "smx_gemm_tf32x3_splits": (_int, [_i64, _int, _int]),
    "smx_gemm_tf32x3_splitk": (_int, [_p, _p, _i64, _p, _p, _i64, _int, _int, _int, _p, _i64, _p, _int, _int, _p, _sz,
                                       _p, _p]),
    "smx_spectral_panel_t_workspace": (_sz, [_int, _i64]),
    "smx_spectral_panel_t_tf32": (_int, [_int, _p, _p, _p, _int, _p, _int, _p, _p, _p, _p, _i64, _i64, _p, _p,
                                          _i64, _p, _sz, _p]),
    "smx_spectral_vjp_x_workspace": (_sz, [_int, _int, _i64]),
    "smx_spectral_vjp_x": (_int, [_int, _p, _p, _p, _int, _p, _int, _p, _int, _p, _p, _p, _p, _i64, _i64, _p, _i64,
                                   _p, _i64, _p, _sz, _p]),
    "smx_spectral_coefficients_adjoint": (_int, [_p, _p, _p, _p, _p, _p, _p]),
    "smx_split_tf32": (_int, [_p, _i64, _i64, _i64, _p, _p, _i64, _p]),
    "smx_layout_build": (_int, [_int, _i64, _p, _p, _p, _p, _p, _p, _p, _int, _p, _int, _p, _p, _p,
                                 C.POINTER(_p)]),
    "smx_layout_build_f64": (_int, [_int, _i64, _p, _p, _p, _p, _p, _p, _p, _int, _p, _int, _p, _p, _p,
                                     C.POINTER(_p)]),
    "smx_fp32_plan_has_fp64": (_int, [_p]),
    "smx_fp32_eval64": (_int, [_p, _p, _i64, _i64, _p, _p]),
    "smx_layout_i32": (_int, [_p, C.c_char_p, C.POINTER(_p), C.POINTER(_i64)]),
    "smx_layout_f32": (_int, [_p, C.c_char_p, C.POINTER(_p), C.POINTER(_i64)]),
    "smx_layout_f64": (_int, [_p, C.c_char_p, C.POINTER(_p), C.POINTER(_i64)]),
    "smx_layout_scalar": (_int, [_p, C.c_char_p, C.POINTER(_dbl)]),
    "smx_layout_free": (None, [_p]),
    "smx_fp32_plan_create": (_int, [_p, _p, _p, _p, _p, _dbl, C.POINTER(_p), _p]),
    "smx_fp32_plan_destroy": (None, [_p]),
    "smx_fp32_plan_info": (_int, [_p, C.POINTER(_int), C.POINTER(_i64), C.POINTER(_p)]),
    "smx_fp32_workspace": (_sz, [_p, _i64]),
    "smx_fp32_eval": (_int, [_p, _p, _i64, _i64, _p, _p, _sz, _p]),
    "smx_fp32_plan_check": (_int, [_p, _p]),
    "smx_vjp_workspace": (_sz, [_p, _i64]),
    "smx_vjp": (_int, [_p, _p, _i64, _i64, _p, _i64, _p, _i64, _p, _p, _sz, _p]),
    "smx_last_error_string": (C.c_char_p, []),
    "smx_version": (C.c_char_p, []),
}

_lib = None


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "smolyax_gb300 CUDA library not built (%s missing); run `python -m smolyax_gb300.build`" % LIB_PATH
        )
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class SmxError(RuntimeError):
    pass


def call(name, *args):
    """Call an entry point returning a status code; raise SmxError on failure."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != SMX_OK:
        msg = lib.smx_last_error_string()
        raise SmxError("%s failed (%d): %s" % (name, rc, msg.decode() if msg else ""))
    return rc


def size(name, *args):
    return int(getattr(load(), name)(*args))


def ptr(t):
    """Device (or host) address of a torch tensor, None for None."""
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_ptr(stream):
    return C.c_void_p(stream.cuda_stream) if stream is not None else None


LAYOUT_KINDS = {"blocked": 0, "perpoint": 1, "tape": 2, "blocked_tc": 3}


def host_layout(kind, tree, coef, d_out, maxdeg, fam, fa, fb, i32=(), f32=(), scalars=(), fp64=False):
    """Tables of the library's host-side layout builder (``smx_layout_build``)
    as numpy copies: {name: array or float}.  ``tree`` holds host arrays
    parent, dim, deg, level, rank, rem; coef is FP32 [n, d_out] (unused for
    the tape).  With ``fp64`` the per-point layout is built with FP64
    coefficients (``smx_layout_build_f64``) and the ``f32`` names are read as
    FP64 tables.  Returns None if the plan is outside the evaluator's limits."""
    import numpy as np

    lib = load()
    n = int(tree["parent"].shape[0])
    d = int(np.asarray(maxdeg).shape[0])
    arr = lambda a, dt: np.ascontiguousarray(np.asarray(a), dtype=dt)
    keep = [arr(tree["parent"], np.int32), arr(tree["dim"], np.int32), arr(tree["deg"], np.int32),
            arr(tree["level"], np.int32), arr(tree["rank"], np.int64), arr(tree["rem"], np.float64),
            arr(coef if coef is not None else np.zeros((n, d_out)), np.float64 if fp64 else np.float32),
            arr(maxdeg, np.int64),
            arr(fam, np.int32), arr(fa, np.float64), arr(fb, np.float64)]
    ptrs = [k.ctypes.data_as(C.c_void_p) for k in keep]
    h = C.c_void_p()
    build = lib.smx_layout_build_f64 if fp64 else lib.smx_layout_build
    rc = build(LAYOUT_KINDS[kind], n, *ptrs[:7], int(d_out), ptrs[7], d, *ptrs[8:], C.byref(h))
    if rc == -5:
        return None
    if rc != SMX_OK:
        raise RuntimeError("smx_layout_build failed (%d): %s" % (rc, lib.smx_last_error_string().decode()))
    out = {}
    try:
        for names, fn, ct, dt in ((i32, lib.smx_layout_i32, C.c_int32, np.int32),
                                  (f32, lib.smx_layout_f64, C.c_double, np.float64) if fp64 else
                                  (f32, lib.smx_layout_f32, C.c_float, np.float32)):
            for name in names:
                p, cnt = C.c_void_p(), _i64()
                if fn(h, name.encode(), C.byref(p), C.byref(cnt)) != SMX_OK:
                    raise KeyError(name)
                out[name] = np.zeros(0, dt) if cnt.value == 0 else \
                    np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(cnt.value,)).astype(dt).copy()
        for name in scalars:
            v = _dbl()
            if lib.smx_layout_scalar(h, name.encode(), C.byref(v)) != SMX_OK:
                raise KeyError(name)
            out[name] = v.value
    finally:
        lib.smx_layout_free(h)
    return out
