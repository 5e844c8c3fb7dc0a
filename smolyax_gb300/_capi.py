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
    "smx_spectral_coefficients": (_int, [_p, _p, _p, _p, _p, _p, _p, _i64, _p, _p, _p, _p, _p]),
    "smx_spectral_eval": (_int, [_p, _p, _i64, _i64, _p, _p]),
    "smx_blocked_smem": (_sz, [_p]),
    "smx_gemm_bf16x3": (_int, [_p, _p, _i64, _p, _p, _i64, _int, _int, _int, _p, _i64, _p, _int, _p, _p]),
    "smx_split_bf16": (_int, [_p, _i64, _i64, _i64, _p, _p, _i64, _p]),
    "smx_host_device_pointer": (_int, [_p, _p]),
    "smx_blocked_eval": (_int, [_p, _p, _i64, _i64, _p, _p, _sz, _p]),
    "smx_blocked_eval_workspace": (_sz, [_p, _i64]),
    "smx_blocked_eval_batch_workspace": (_sz, [_int, _int]),
    "smx_blocked_eval_batch": (_int, [_p, _int, _p, _int, _p, _sz, _p]),
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
    "smx_gemm_tf32x3_splitk": (_int, [_p, _p, _i64, _p, _p, _i64, _int, _int, _int, _p, _i64, _p, _int, _int, _p, _sz,
                                       _p, _p]),
    "smx_spectral_panel_t_workspace": (_sz, [_int, _i64]),
    "smx_spectral_panel_t_tf32": (_int, [_int, _p, _p, _p, _int, _p, _int, _p, _p, _p, _p, _i64, _i64, _p, _p,
                                          _i64, _p, _sz, _p]),
    "smx_spectral_vjp_x_workspace": (_sz, [_int, _i64]),
    "smx_spectral_vjp_x": (_int, [_int, _p, _p, _p, _int, _p, _int, _p, _p, _p, _p, _i64, _i64, _p, _i64, _p, _i64,
                                   _p, _sz, _p]),
    "smx_spectral_coefficients_adjoint": (_int, [_p, _p, _p, _p, _p, _p, _p]),
    "smx_split_tf32": (_int, [_p, _i64, _i64, _i64, _p, _p, _i64, _p]),
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
