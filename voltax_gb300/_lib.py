"""ctypes binding of ``libvxg.so`` (the C ABI declared in include/vxg.h).

The library is loaded from ``voltax_gb300/_lib/``; it is built in-tree by
``voltax_gb300.build``. There is no CPU fallback: if the library or a CUDA
device is missing, every GPU entry point raises.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libvxg.so"

VXG_OK, VXG_ERR_INVALID, VXG_ERR_CUDA, VXG_ERR_TOO_LARGE, VXG_ERR_ALLOC = range(5)
VXG_F64, VXG_F32, VXG_C128 = 0, 1, 2
VXG_MODE_DC, VXG_MODE_BE, VXG_MODE_TRAP = 0, 1, 2
VXG_ACT_NONE, VXG_ACT_GELU = 0, 1
MAX_GROUPS = 32

_ERRORS = {VXG_ERR_INVALID: "invalid argument", VXG_ERR_CUDA: "CUDA error",
           VXG_ERR_TOO_LARGE: "supernode too large for the shared-memory kernels",
           VXG_ERR_ALLOC: "allocation failed"}

P = C.c_void_p
I32, I64, F64 = C.c_int32, C.c_int64, C.c_double
PI32, PI64, PF64 = C.POINTER(I32), C.POINTER(I64), C.POINTER(F64)


class GroupDesc(C.Structure):
    _fields_ = [("kind", I32), ("n", I32), ("T", I32), ("K", I32), ("wave", I32),
                ("n_params", I32), ("int_offset", I32), ("nodes", PI32)]


class TopologyDesc(C.Structure):
    _fields_ = [
        ("size", I32), ("n_nodes", I32), ("nnz", I64),
        ("indptr", PI64), ("indices", PI32), ("rows", PI32), ("tptr", PI64), ("tent", PI64),
        ("diag", PI64), ("n_groups", I32), ("groups", C.POINTER(GroupDesc)),
        ("n_res_slots", I64), ("res_ptr", PI64), ("res_src", PI64),
        ("n_jac_slots", I64), ("jac_ptr", PI64), ("jac_src", PI64),
        ("n_seg", I32), ("seg_ptr", PI32), ("seg_of", PI32), ("seg_idx", PI32),
        ("n_sn", I32), ("sn_k", PI32), ("sn_r", PI32), ("sn_panel", PI64),
        ("sn_piv_ptr", PI64), ("sn_piv", PI32), ("sn_bord_ptr", PI64), ("sn_bord", PI32),
        ("work", I64), ("a_pos", PI64),
        ("n_levels", I32), ("lv_ptr", PI64), ("lv_sn", PI32), ("lv_schur_off", PI64),
        ("lv_bord_off", PI64), ("lv_schur_len", PI64), ("lv_bord_len", PI64),
        ("lv_st_ptr", PI64), ("st_tgt", PI64), ("st_ptr", PI64), ("st_src", PI64),
        ("lv_bt_ptr", PI64), ("bt_tgt", PI32), ("bt_ptr", PI64), ("bt_src", PI64),
    ]


class GroupParams(C.Structure):
    _fields_ = [("params", P), ("row_stride", I64), ("batch_stride", I64)]


class NewtonOpts(C.Structure):
    _fields_ = [("max_steps", I32), ("rtol", F64), ("atol", F64), ("max_dv", F64),
                ("precision", I32), ("refine", I32), ("block", I32)]


SIGNATURES = {
    "vxg_last_error": ([], C.c_char_p),
    "vxg_create": ([C.POINTER(TopologyDesc), C.POINTER(P)], I32),
    "vxg_destroy": ([P], I32),
    "vxg_workspace_size": ([P, I32, I32, C.POINTER(C.c_size_t)], I32),
    "vxg_factor_size": ([P, I32, I32, C.POINTER(C.c_size_t)], I32),
    "vxg_eval": ([P, I32, C.POINTER(GroupParams), P, F64, F64, F64, P, F64, P, P, P, P, P],
                 I32),
    "vxg_factor": ([P, I32, I32, P, P, P, P], I32),
    "vxg_solve": ([P, I32, I32, P, P, P, P, I32, I32, P, P], I32),
    "vxg_spmv": ([P, I32, P, P, P, I32, P], I32),
    "vxg_level_count": ([P, C.POINTER(I32)], I32),
    "vxg_tune_factor": ([P, I32, I32, P, P, P, P, P], I32),
    "vxg_set_factor_shapes": ([P, I32, P], I32),
    "vxg_spsolve_gdata": ([P, I32, P, P, P, P], I32),
    "vxg_newton": ([P, I32, C.POINTER(GroupParams), I32, F64, F64, P, P, F64,
                    C.POINTER(NewtonOpts), P, P, P, P, P, P], I32),
    "vxg_newton_masked": ([P, I32, C.POINTER(GroupParams), I32, F64, F64, P, P, F64,
                           C.POINTER(NewtonOpts), P, P, P, P, P, P], I32),
    "vxg_transient": ([P, I32, C.POINTER(GroupParams), I32, I32, PF64, P, F64,
                       C.POINTER(NewtonOpts), P, P, P, P, P], I32),
    "vxg_fused_smem": ([P, I32, C.POINTER(C.c_size_t)], I32),
    "vxg_fused_run": ([P, I32, C.POINTER(GroupParams), I32, I32, P, P, I32, P, I32, I32, F64,
                       C.POINTER(NewtonOpts), P, P, P, P], I32),
    "vxg_fused_sweep": ([P, I32, C.POINTER(GroupParams), I32, I32, I32, I32, P, F64, P, P, I32,
                         I32, F64, C.POINTER(NewtonOpts), P, P, P, P], I32),
    "vxg_factor_static": ([P, I32, I32, P, P, P], I32),
    "vxg_gemm_tf32x3": ([I32, I32, I32, P, I32, P, I32, P, I32, P, P], I32),
    "vxg_fused_set_profile": ([P], I32),
    "vxg_launch_count": ([], C.c_uint64),
    "vxg_ac_factor": ([P, I32, P, P, P, P, P, P], I32),
    "vxg_ac_solve": ([P, I32, P, P, I64, P, P, P], I32),
    "vxg_mlp_normalize": ([I64, I32, P, I64, P, P, P, P, P], I32),
    "vxg_mlp_linear": ([I64, I32, I32, P, P, P, I32, P, P, P, P, P, P, I64, P], I32),
    "vxg_mlp_linear_dx": ([I64, I32, I32, P, P, P, P, P], I32),
    "vxg_mlp_linear_dw": ([I64, I32, I32, P, P, P, P, P], I32),
    "vxg_mlp_mse": ([I64, I32, P, P, P, P, P, P, P], I32),
    "vxg_mlp_adam": ([I64, P, P, P, P, P, C.c_float, C.c_float, C.c_float, C.c_float, I32, P],
                     I32),
    "vxg_param_vjp": ([P, I32, C.POINTER(GroupParams), P, F64, F64, F64, P,
                       C.POINTER(P), P], I32),
}

_lib = None


class VxgError(RuntimeError):
    pass


def load() -> C.CDLL:
    """Load ``libvxg.so`` (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise VxgError(f"{LIB_PATH} is missing: build it with "
                           "`python -m voltax_gb300.build` (there is no CPU fallback)")
        lib = C.CDLL(str(LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def check(status: int, what: str) -> None:
    if status != VXG_OK:
        detail = load().vxg_last_error().decode()
        raise VxgError(f"{what} failed: {_ERRORS.get(status, status)} {detail}".strip())


def exported_symbols() -> list[str]:
    return list(SIGNATURES)
