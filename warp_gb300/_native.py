"""ctypes bindings to ``libwarp_gb300.so`` (the sm_103a CUDA library).

The library is built in-tree by ``warp_gb300._build.build()`` (``__graft_entry__.build()`` calls
it).  There is no fallback: if the library is missing every entry point raises, loudly.
"""

from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libwarp_gb300.so")

GB_F32, GB_F64, GB_BF16, GB_F16 = 0, 1, 2, 3
KRYLOV_CG, KRYLOV_BICGSTAB, KRYLOV_FCG = 0, 1, 2

# z = M(r) callback of the flexible solver: (user, stream, r, z) -> status
PRECOND_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)

# device status bits
DEV_WAIT_TIMEOUT = 1
DEV_BREAKDOWN = 2
DEV_NONFINITE = 4
DEV_STAGNATION = 8

_c_int, _c_i64, _c_u64, _c_sz, _c_dbl = ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_double
_vp = ctypes.c_void_p

# name -> (restype, argtypes); mirrors include/warp_gb300.h
_SIGNATURES = {
    "gb_last_error": (ctypes.c_char_p, []),
    "gb_clear_error": (None, []),
    "gb_version": (_c_int, []),
    "gb_set_pdl": (_c_int, [_c_int]),
    "gb_get_pdl": (_c_int, []),
    "gb_device_arch": (_c_int, []),
    "gb_scan_i32_workspace_bytes": (_c_sz, [_c_i64]),
    "gb_scan_i32": (_c_int, [_vp, _vp, _c_i64, _c_int, _vp, _c_sz, _vp]),
    "gb_scan_i32_noalloc_max_n": (_c_i64, []),
    "gb_scan_i32_noalloc": (_c_int, [_vp, _vp, _c_i64, _c_int, _vp]),
    "gb_bsr_from_triplets_workspace_bytes": (_c_sz, [_c_int, _c_int, _c_int]),
    "gb_bsr_matrix_from_triplets_device": (
        _c_int,
        [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_u64, _c_int, _vp, _vp, _vp, _vp, _vp, _vp,
         _vp, _vp, _c_sz, _vp],
    ),
    "gb_bsr_accumulate_triplet_values": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _c_int, _vp]),
    "gb_bsr_mv": (
        _c_int,
        [_c_int, _c_int, _c_int, _c_int, _c_i64, _c_i64, _vp, _vp, _vp, _vp, _c_int, _vp, _vp, _vp, _c_int, _c_dbl,
         _c_dbl, _c_int, _c_int, _c_int, _c_int, _vp, _vp],
    ),
    "gb_bsr_mv_default_shape": (_c_int, [_c_int, _c_int, _c_int, _c_int, _c_i64, _vp, _vp, _vp]),
    "gb_krylov_workspace_bytes": (_c_sz, [_c_int, _c_int, _c_int, _c_i64, _c_int]),
    "gb_krylov_create": (_c_int, [_c_int, _c_int, _c_int, _c_i64, _c_i64, _c_int, _c_int, _c_int, _c_int, _vp, _c_sz,
                                  ctypes.POINTER(_vp)]),
    "gb_krylov_destroy": (_c_int, [_vp]),
    "gb_krylov_set_operands": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_int, _c_dbl, _c_dbl, _c_int,
                                        _c_int, _vp]),
    "gb_krylov_launch": (_c_int, [_vp, _c_int, _c_int, _vp]),
    "gb_krylov_scalars": (_c_int, [_vp, _vp, _vp, _vp, _vp]),
    "gb_krylov_read": (_c_int, [_vp, _vp, _vp, _vp]),
    "gb_krylov_vectors": (_c_int, [_vp, _vp, _vp, _vp]),
    "gb_residual_f64_workspace_bytes": (_c_sz, [_c_int, _c_int, _c_i64, _c_int]),
    "gb_residual_f64": (_c_int, [_c_int, _c_int, _c_i64, _c_i64, _vp, _vp, _vp, _vp, _c_int, _vp, _vp, _vp, _vp,
                                 _vp, _vp, _c_sz, _vp, _vp]),
    "gb_axpy_f64_f32": (_c_int, [_c_i64, _vp, _vp, _c_dbl, _vp]),
    "gb_residual_df": (_c_int, [_c_int, _c_int, _c_i64, _c_i64, _vp, _vp, _vp, _vp, _c_int, _vp, _vp, _vp, _vp,
                                _vp, _vp, _c_sz, _vp, _vp]),
    "gb_update_solution": (_c_int, [_c_i64, _vp, _vp, _vp, _c_dbl, _vp]),
    "gb_krylov_set_precond": (_c_int, [_vp, _vp, _vp, _c_int, _c_dbl]),
    "gb_krylov_set_persistent": (_c_int, [_vp, _c_int, _vp]),
    "gb_krylov_set_stencil": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp]),
    "gb_bsr_jacobi_smooth": (_c_int, [_c_int, _c_int, _c_i64, _c_i64, _vp, _vp, _vp, _c_int, _vp, _vp, _vp,
                                      ctypes.c_float, _vp, _vp, _vp]),
    "gb_mg_restrict": (_c_int, [_c_int] * 6 + [_vp, _vp, _vp, _vp, _vp]),
    "gb_mg_restrict_c": (_c_int, [_c_int] * 7 + [_vp, _vp, _vp, _vp, _vp]),
    "gb_mg_prolong_add_c": (_c_int, [_c_int] * 7 + [_vp, _vp, ctypes.c_float, _vp, _vp]),
    "gb_mg_prolong_add": (_c_int, [_c_int] * 6 + [_vp, _vp, ctypes.c_float, _vp, _vp]),
    "gb_mg_jacobi0": (_c_int, [_c_i64, ctypes.c_float, _vp, _vp, _vp, _vp]),
    "gb_bsr_block_inverse_diagonal3": (_c_int, [_c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gb_mg_block_jacobi0": (_c_int, [_c_i64, ctypes.c_float, _vp, _vp, _vp, _vp]),
    "gb_bsr_block_jacobi_smooth3": (_c_int, [_c_int, _c_i64, _c_i64, _vp, _vp, _vp, _c_int, _vp, _vp, _vp,
                                             ctypes.c_float, _vp, _vp, _vp]),
    "gb_st27_bytes": (_c_sz, [_c_int, _c_int, _c_int]),
    "gb_st27_build": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gb_st27_apply": (_c_int, [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, ctypes.c_float, _vp, _vp, _vp, _vp]),
    "gb_st27_bytes_bf16": (_c_sz, [_c_int, _c_int, _c_int]),
    "gb_residual_df_st27": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_sz, _vp, _vp]),
    "gb_st27_to_bf16": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp]),
    "gb_st27_apply_bf16": (_c_int, [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, ctypes.c_float, _vp, _vp, _vp,
                                    _vp]),
    "gb_mg_coarsen_cells": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp]),
    "gb_bsr_get_diag": (_c_int, [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gb_bsr_inverse_diagonal": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int, _vp, _vp]),
    "gb_diag_mv": (_c_int, [_c_int, _c_i64, _vp, _vp, _vp, _vp, _c_dbl, _c_dbl, _vp]),
    "gb_dense_mv": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_dbl, _c_dbl, _vp]),
    "gb_dots_workspace_bytes": (_c_sz, []),
    "gb_dots": (_c_int, [_c_int, _c_i64, _c_int, ctypes.POINTER(_vp), ctypes.POINTER(_vp), _vp, _vp, _vp]),
    "gb_axpby": (_c_int, [_c_int, _c_i64, _c_dbl, _vp, _c_dbl, _vp, _vp, _vp]),
    "gb_conv3_fwd_f32": (_c_int, [_c_int] * 5 + [_vp, _vp, _c_int, _vp, _vp]),
    "gb_conv3_bwd_data_f32": (_c_int, [_c_int] * 5 + [_vp, _vp, _vp, _vp]),
    "gb_conv3_bwd_weight_workspace_bytes": (_c_sz, [_c_int] * 5),
    "gb_conv3_bwd_weight_f32": (_c_int, [_c_int] * 5 + [_vp, _vp, _vp, _vp, _c_sz, _vp]),
    "gb_relu_bwd": (_c_int, [_c_i64, _vp, _vp, _vp]),
    "gb_adam_step": (_c_int, [_c_int, _vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                              ctypes.c_float, _c_int, _vp, _vp]),
    "gb_net_features": (_c_int, [_c_int, _c_int, _c_i64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gb_net_cell_features": (_c_int, [_c_int, _c_int, _c_int, _vp, ctypes.c_float, ctypes.c_float, _vp, _vp]),
    "gb_net_combine": (_c_int, [_c_int, _c_int, _c_i64, _c_int, _vp, _vp, ctypes.c_float, _vp, _vp, _vp, _vp]),
    "gb_conv3_planar_rows": (_c_i64, [_c_int] * 3),
    "gb_net_features_planar": (_c_int, [_c_int] * 4 + [_vp, _vp, _vp, _vp, _vp, _vp]),
    "gb_conv3_fwd_tc": (_c_int, [_c_int] * 4 + [_vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_float, _vp, _vp]),
    "gb_convnet_tc_items": (_c_i64, [_c_int] * 3),
    "gb_convnet_fwd_tc": (_c_int, [_c_int] * 5 + [_vp] * 7 + [ctypes.c_float, _vp, _vp, _vp, _vp]),
    "gb_batched_pcg_workspace_bytes": (_c_sz, [_c_i64]),
    "gb_batched_pcg": (_c_int, [_c_int, _vp, _vp, _c_i64, _vp, _vp, _vp, _vp, _vp, _vp, _c_dbl, _c_dbl, _c_int, _c_int,
                                _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_sz, _vp, _vp]),
    "gb_batched_bicgstab_workspace_bytes": (_c_sz, [_c_i64]),
    "gb_batched_bicgstab": (_c_int, [_c_int, _vp, _vp, _c_i64, _vp, _vp, _vp, _vp, _vp, _vp, _c_dbl, _c_dbl, _c_int,
                                     _c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_sz, _vp, _vp]),
    "gb_batched_pcg2": (_c_int, [_c_int, _vp, _vp, _c_i64, _vp, _vp, _vp, _vp, _vp, _vp, _c_dbl, _c_dbl, _c_int,
                                 _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_sz, _vp, _vp]),
    "gb_multi_dot_workspace_bytes": (_c_sz, [_c_int]),
    "gb_multi_dot": (_c_int, [_c_int, _c_i64, _c_int, _vp, _c_i64, _vp, _vp, _vp, _c_sz, _vp]),
    "gb_multi_axpy": (_c_int, [_c_int, _c_i64, _c_int, _vp, _c_i64, _vp, _c_dbl, _c_dbl, _vp, _vp]),
    "gb_bsr_scatter_padded": (_c_int, [_c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gb_bsr_gather_blocks": (_c_int, [_c_int, _c_int, _c_i64, _vp, _vp, _vp, _vp]),
    "gb_bsr_rows_to_offsets": (_c_int, [_c_i64, _vp, _c_int, _vp, _vp, _vp]),
    "gb_bsr_compress_rows": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int, _c_u64, _vp, _vp]),
    "gb_bsr_compact_workspace_bytes": (_c_sz, [_c_int]),
    "gb_bsr_compact": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_sz, _vp]),
    "gb_q1_batched_assemble_2d": (_c_int, [_c_int, _vp, _vp, _vp, _vp, _vp, _vp, _c_int, _vp, _vp, _vp, _vp, _vp]),
}

_LIB = None


def exported_names() -> list[str]:
    return sorted(_SIGNATURES)


def register(name: str, restype, argtypes) -> None:
    """Declare one more entry point (used by modules that add C-ABI functions)."""
    _SIGNATURES[name] = (restype, argtypes)
    if _LIB is not None:
        f = getattr(_LIB, name)
        f.restype, f.argtypes = restype, argtypes


def lib():
    """Load the CUDA library; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"warp_gb300 CUDA library not found at {LIB_PATH}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)"
            )
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _LIB = L
    return _LIB


class GbError(RuntimeError):
    pass


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = lib().gb_last_error().decode(errors="replace")
        raise GbError(f"{what}: {msg} (status {rc})" if what else f"{msg} (status {rc})")


def call(name: str, *args):
    rc = getattr(lib(), name)(*args)
    check(rc, name)
    return rc
