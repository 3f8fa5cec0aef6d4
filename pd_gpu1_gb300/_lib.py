"""ctypes binding of libpd_gb300.so (the C ABI declared in include/pd.h).

The library is loaded from this package's directory.  There is no fallback:
if the shared object is missing or fails to load, importing any entry point
raises, so a run without the CUDA engine cannot pass silently.
"""
import ctypes as C
import os

from ._abi import PDCylinder, PDLoadStepStats, PDParams, PDResult, PDSpecimen

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpd_gb300.so")

_lib = None

P = C.POINTER
VP = C.c_void_p
D = C.c_double
I32 = C.c_int
I64 = C.c_int64
SZ = C.c_size_t

_SIGS = {
    "pd_status_string": (C.c_char_p, [I32]),
    "pd_last_error": (C.c_char_p, [VP]),
    "pd_params_derive": (I32, [P(PDParams), I32, I32, I32] + [D] * 12 + [I32]),
    "pd_create": (VP, [P(PDParams), P(I32)]),
    "pd_destroy": (I32, [VP]),
    "pd_debug_fail_allocation": (I32, [I32]),
    "pd_get_params": (I32, [VP, P(PDParams)]),
    "pd_set_params": (I32, [VP, P(PDParams)]),
    "pd_get_field": (I32, [VP, I32, VP, SZ, VP]),
    "pd_set_field": (I32, [VP, I32, VP, SZ, VP]),
    "pd_field_ptr": (I32, [VP, I32, P(VP), P(SZ)]),
    "pd_count_broken": (I32, [VP, P(I64), VP]),
    "pd_num_bonds": (I64, [VP]),
    "pd_sync": (I32, [VP, VP]),
    "pd_coord_plate": (I32, [VP, VP]),
    "pd_coord_plate_crack": (I32, [VP, VP]),
    "pd_coord_kw": (I32, [P(PDParams), D, P(D), P(D), P(D), I64, P(I64)]),
    "pd_find_neighbor": (I32, [VP, VP]),
    "pd_vol_corr": (I32, [VP, VP]),
    "pd_surface_correct": (I32, [VP, VP]),
    "pd_initial_weight": (I32, [VP, VP]),
    "pd_set_crack_2d": (I32, [VP, D, D, D, D, VP]),
    "pd_set_crack_kw": (I32, [VP, D, VP]),
    "pd_initial_state": (I32, [VP, VP]),
    "pd_prepare": (I32, [VP, VP]),
    "pd_bond_force": (I32, [VP, VP]),
    "pd_state_force": (I32, [VP, VP]),
    "pd_integrate_adr": (I32, [VP, I32, VP]),
    "pd_get_adr_cn": (I32, [VP, P(D), VP]),
    "pd_integrate_verlet1": (I32, [VP, VP]),
    "pd_integrate_verlet2": (I32, [VP, VP]),
    "pd_reduce_sum": (I32, [VP, VP, I64, P(D), VP]),
    "pd_damage": (I32, [VP, VP]),
    "pd_quick_load": (I32, [VP, D, VP]),
    "pd_load_plate_tensile": (I32, [VP, VP]),
    "pd_cylinder_init": (I32, [VP, P(PDCylinder), VP]),
    "pd_cylinder_get": (I32, [VP, P(PDCylinder), VP]),
    "pd_cylinder_integrate1": (I32, [VP, VP]),
    "pd_contact": (I32, [VP, VP]),
    "pd_cylinder_integrate2": (I32, [VP, VP]),
    "pd_run_adr": (I32, [VP, I32, I32, D, VP]),
    "pd_run_explicit": (I32, [VP, I32, D, I32, VP]),
    "pd_residual": (I32, [VP, P(D), VP]),
    "pd_adr_solve": (I32, [VP, I32, I32, I32, D, P(I32), P(D), VP]),
    "pd_load_step": (I32, [VP, D, VP, I32, I32, D, I32, I32, P(PDLoadStepStats), VP]),
    "pd_mlp_create": (VP, [I64, P(I32)]),
    "pd_mlp_destroy": (I32, [VP]),
    "pd_mlp_num_params": (I32, []),
    "pd_mlp_set_params": (I32, [VP, VP, I64]),
    "pd_mlp_get_params": (I32, [VP, VP, I64]),
    "pd_mlp_forward": (I32, [VP, VP, I64, VP, VP]),
    "pd_mlp_forward_layers": (I32, [VP, VP, I64, VP, VP]),
    "pd_mlp_grad": (I32, [VP, VP, VP, I64, VP, P(C.c_float), VP]),
    "pd_mlp_train_step": (I32, [VP, VP, VP, I64, C.c_float, P(C.c_float), VP]),
    "pd_mlp_gemm": (I32, [VP, VP, I64, I64, I64, VP, I32, VP]),
    "pd_mlp_gemm_wait_check": (I32, [VP, VP, I64, I64, I64, VP, I32, C.c_longlong, I32, VP]),
    "pd_warm_features": (I32, [VP, D, D, VP, VP]),
    "pd_warm_record": (I32, [VP, D, D, VP, VP, VP]),
    "pd_warm_predict": (I32, [VP, VP, D, D, I32, VP, VP]),
    "pd_batch_create": (VP, [P(PDParams), P(PDSpecimen), I32, P(I32)]),
    "pd_batch_info": (I32, [VP, P(I32), P(I64), P(I64)]),
    "pd_batch_run_adr": (I32, [VP, I32, I32, D, VP]),
    "pd_batch_get_cn": (I32, [VP, P(D), VP]),
    "pd_set_launch": (I32, [VP, I32, I32, I32, I32]),
    "pd_get_launch": (I32, [VP, P(I32), P(I32), P(I32), P(I32)]),
    "pd_set_force_layout": (I32, [VP, I32]),
    "pd_get_force_layout": (I32, [VP, P(I32)]),
    "pd_autotune": (I32, [VP, I32, P(D), VP]),
    "pd_profile_steps": (I32, [VP, I32, I32, I32, D, P(D), P(D), VP]),
    "pd_solve_plate_tensile": (I32, [D, I32, P(D), P(D), P(D), P(PDResult)]),
    "pd_solve_plate_crack_grow": (I32, [D, I32, P(D), P(D), P(D), P(PDResult)]),
    "pd_solve_kalthoff_winkler": (I32, [D, I32, P(D), P(D), P(D), P(D), I64, P(PDResult)]),
    "pd_write_disp_txt": (I32, [C.c_char_p, I64, VP, VP, VP, VP]),
    "pd_write_kw_txt": (I32, [C.c_char_p, P(PDParams), D, I64, VP, VP, VP, VP]),
    "pd_save_disp": (I32, [VP, C.c_char_p, VP]),
    "pd_save_kw": (I32, [VP, D, C.c_char_p, VP]),
    "pd_snapshot_save": (I32, [VP, C.c_char_p, VP]),
    "pd_snapshot_load": (I32, [VP, C.c_char_p, VP]),
    "pd_crack_tip": (I32, [VP, D, P(D), VP]),
    "pd_check_finite": (I32, [VP, VP]),
    "pd_kernel_launches": (I64, [VP]),
    "pd_probe_fp64": (I32, [P(D)]),
    "pd_check_division": (I32, [VP, VP, I64, VP, VP]),
    "pd_reduce_sum_static": (I32, [VP, I64, VP, VP]),
}


def exported_symbols():
    """Names the C ABI exports (as declared in include/pd.h)."""
    return list(_SIGS)


def lib():
    """Load libpd_gb300.so; raises if it is missing (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        handle = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


class PDError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def check(status, ctx=None, what=""):
    if status != 0:
        L = lib()
        name = L.pd_status_string(status).decode()
        detail = L.pd_last_error(ctx).decode() if ctx else ""
        raise PDError(status, f"{what}: {name} {detail}".strip())
    return status
