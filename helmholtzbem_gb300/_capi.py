"""ctypes binding of libhbem.so (include/hbem.h).

The library is the only compute path: if it is missing or fails to load this
module raises, so nothing silently falls back to CPU code.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libhbem.so")

HBEM_OK = 0
LAYER_DOUBLE, LAYER_SINGLE, LAYER_HYPERSINGULAR, LAYER_ALL = 1, 2, 4, 7
PANEL_LINE, PANEL_ARC = 0, 1
SPACE_P0, SPACE_P1 = 1, 2

# every symbol include/hbem.h declares
EXPORTS = [
    "hbem_version", "hbem_status_string", "hbem_last_error", "hbem_set_device", "hbem_set_option", "hbem_get_option",
    "hbem_hankel01",
    "hbem_stats_enable_timing", "hbem_stats_reset", "hbem_stats_read", "hbem_stats_read_points",
    "hbem_builder_create", "hbem_builder_destroy", "hbem_builder_info", "hbem_builder_is_adjacent",
    "hbem_assemble_dense", "hbem_assemble_dense_sub", "hbem_get_layer", "hbem_get_layer_device",
    "hbem_solop_create", "hbem_solop_destroy", "hbem_mass_matrix", "hbem_gen_sol_op",
    "hbem_gen_sol_op_batch_device", "hbem_gen_sol_op_multi_device", "hbem_sv_dense_batch_device", "hbem_sv_dense_batch_noalloc",
    "hbem_sv_dense_batch", "hbem_sweep_sigma", "hbem_rand_sketch", "hbem_rsvd_sv_batch",
    "hbem_rsvd_sv_batch_device", "hbem_rsvd_sv_batch_device_ex", "hbem_lu_factor_batch_device", "hbem_lu_solve_batch_device",
    "hbem_cgemm_f32_batch_device", "hbem_lu_factor_batch_device_f32", "hbem_solop_info", "hbem_sigma_rsvd_sweep", "hbem_opt_subdiv",
    "hbem_find_resonances_adaptive", "hbem_arnoldi_sv_batch", "hbem_arnoldi_sv_batch_device",
    "hbem_scatterer_read", "hbem_polygon_length", "hbem_auto_num_panels", "hbem_polygon_panels",
    "hbem_polygon_panels_graded", "hbem_choose_num_panels",
    "hbem_incoming_load", "hbem_incoming_eval", "hbem_tp_solve", "hbem_tp_field_grid", "hbem_field_stats",
    "hbem_mlp_create", "hbem_mlp_destroy", "hbem_mlp_num_params", "hbem_mlp_get_params", "hbem_mlp_set_params",
    "hbem_mlp_forward", "hbem_mlp_gradients", "hbem_mlp_train_step", "hbem_bf16_gemm_device",
    "hbem_refine_brackets", "hbem_sweep_sigma_multi", "hbem_find_resonances_plain_multi", "hbem_refine_brackets_multi",
    "hbem_find_resonances_plain", "hbem_find_resonances_plain_verified", "hbem_rtsafe", "hbem_zbrent", "hbem_brent_min",
    "hbem_brent_rc_create", "hbem_brent_rc_step", "hbem_brent_rc_destroy", "hbem_brent_guess", "hbem_brent_gsl",
    "hbem_brent_gsl_with_values",
]

_lib = None

_d = ctypes.c_double
_i = ctypes.c_int
_u = ctypes.c_uint
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_up = ctypes.POINTER(ctypes.c_uint)
_fp = ctypes.POINTER(ctypes.c_float)

FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_double, ctypes.c_void_p)
FN_BOTH = ctypes.CFUNCTYPE(None, ctypes.c_double, _dp, _dp, ctypes.c_void_p)
FN_BATCH = ctypes.CFUNCTYPE(None, _dp, ctypes.c_int, _dp, ctypes.c_void_p)


class HbemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("hbem status %d (%s): %s" % (status, _status_name(status), msg))
        self.status = status


def _status_name(s):
    try:
        return lib().hbem_status_string(s).decode()
    except Exception:
        return "?"


def load(path=LIB_PATH):
    """Load libhbem.so without touching the GPU (symbol table only)."""
    if not os.path.exists(path):
        raise RuntimeError("libhbem.so is not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    sig = {
        "hbem_version": (_i, []),
        "hbem_status_string": (ctypes.c_char_p, [_i]),
        "hbem_last_error": (ctypes.c_char_p, []),
        "hbem_set_device": (_i, [_i]),
        "hbem_set_option": (_i, [ctypes.c_char_p, _i]),
        "hbem_get_option": (_i, [ctypes.c_char_p, _ip]),
        "hbem_hankel01": (_i, [_i, _dp, _i, _dp, _dp]),
        "hbem_stats_enable_timing": (None, [_i]),
        "hbem_stats_reset": (None, []),
        "hbem_stats_read_points": (None, [ctypes.POINTER(ctypes.c_longlong)]),
        "hbem_stats_read": (None, [ctypes.POINTER(ctypes.c_longlong), _dp, ctypes.POINTER(ctypes.c_longlong),
                                   ctypes.POINTER(ctypes.c_longlong)]),
        "hbem_builder_create": (_i, [_i, _ip, _dp, _i, _i, _i, ctypes.POINTER(_vp)]),
        "hbem_builder_destroy": (_i, [_vp]),
        "hbem_builder_info": (_i, [_vp, _ip, _ip, _ip, _ip, _ip]),
        "hbem_builder_is_adjacent": (_i, [_vp, _i, _i, _ip, _ip]),
        "hbem_assemble_dense": (_i, [_vp, _d, _d, _d, _u, _u]),
        "hbem_assemble_dense_sub": (_i, [_vp, _d, _d, _d, _u, _u, _u, _u, _u, _u]),
        "hbem_get_layer": (_i, [_vp, _u, _u, _dp]),
        "hbem_get_layer_device": (_i, [_vp, _u, _u, ctypes.POINTER(_vp)]),
        "hbem_solop_create": (_i, [_vp, _i, ctypes.POINTER(_vp)]),
        "hbem_solop_destroy": (_i, [_vp]),
        "hbem_mass_matrix": (_i, [_vp, _dp]),
        "hbem_gen_sol_op": (_i, [_vp, _d, _d, _d, _d, _u, _dp]),
        "hbem_gen_sol_op_batch_device": (_i, [_vp, _dp, _i, _d, _d, _u, _vp]),
        "hbem_gen_sol_op_multi_device": (_i, [_vp, _i, _ip, _dp, _dp, _d, _u, ctypes.POINTER(_vp)]),
        "hbem_sv_dense_batch_device": (_i, [_i, _i, _u, _vp, ctypes.c_longlong, ctypes.c_longlong, _dp, _dp]),
        "hbem_sv_dense_batch_noalloc": (_i, [_i, _i, _u, _vp, ctypes.c_longlong, ctypes.c_longlong, _vp, _vp, _vp]),
        "hbem_sv_dense_batch": (_i, [_i, _i, _u, _dp, _dp, _dp]),
        "hbem_sweep_sigma": (_i, [_vp, _dp, _i, _d, _d, _u, _dp]),
        "hbem_rand_sketch": (_i, [_i, _i, ctypes.c_ulonglong, _dp]),
        "hbem_rsvd_sv_batch": (_i, [_i, _i, _u, _dp, _dp, _i, _i, _dp]),
        "hbem_rsvd_sv_batch_device": (_i, [_i, _i, _u, _vp, ctypes.c_longlong, ctypes.c_longlong, _vp, _i, _i,
                                           _dp]),
        "hbem_rsvd_sv_batch_device_ex": (_i, [_i, _i, _u, _vp, ctypes.c_longlong, ctypes.c_longlong, _vp, _i, _i,
                                              _i, _i, _dp]),
        "hbem_scatterer_read": (_i, [ctypes.c_char_p, _d, _dp, _dp, _i, _ip]),
        "hbem_polygon_length": (_d, [_dp, _dp, _i]),
        "hbem_auto_num_panels": (_u, [_dp, _dp, _i, _d]),
        "hbem_polygon_panels": (_i, [_dp, _dp, _i, _u, _dp, _i, _ip]),
        "hbem_polygon_panels_graded": (_i, [_dp, _dp, _i, _u, _d, _dp, _i, _ip]),
        "hbem_choose_num_panels": (_i, [_dp, _dp, _i, _d, _d, _d, _up]),
        "hbem_incoming_load": (_i, [ctypes.c_char_p, _dp, _i, _ip]),
        "hbem_incoming_eval": (_i, [_dp, _i, _d, _d, _dp, _i, _dp, _dp]),
        "hbem_tp_solve": (_i, [_vp, _dp, _i, _d, _d, _d, _d, _dp]),
        "hbem_tp_field_grid": (_i, [_vp, _dp, _i, _d, _d, _d, _d, _u, _d, _d, _d, _d, _i, _i, _i, _dp, _dp, _dp,
                                    _dp]),
        "hbem_field_stats": (None, [_dp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
        "hbem_sweep_sigma_multi": (_i, [_vp, _i, _ip, _dp, _dp, _d, _u, _dp]),
        "hbem_find_resonances_plain_multi": (_i, [_vp, _i, _dp, _dp, _i, _d, _dp, _d, _dp, _i, _ip, _ip]),
        "hbem_refine_brackets_multi": (_i, [_vp, _i, _ip, _dp, _dp, _d, _dp, _d, _i, _dp, _i, _ip, _ip]),
        "hbem_refine_brackets": (_i, [_vp, _dp, _dp, _i, _d, _d, _d, _i, _dp, _i, _ip, _ip]),
        "hbem_mlp_create": (_i, [_i, _i, _i, _i, ctypes.c_ulonglong, ctypes.POINTER(_vp)]),
        "hbem_mlp_destroy": (_i, [_vp]),
        "hbem_mlp_num_params": (_i, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
        "hbem_mlp_get_params": (_i, [_vp, _fp]),
        "hbem_mlp_set_params": (_i, [_vp, _fp]),
        "hbem_mlp_forward": (_i, [_vp, _fp, _i, _fp]),
        "hbem_mlp_gradients": (_i, [_vp, _fp, _fp, _i, _fp, _fp]),
        "hbem_mlp_train_step": (_i, [_vp, _fp, _fp, _i, ctypes.c_float, _fp]),
        "hbem_bf16_gemm_device": (_i, [_i, _i, _i, _vp, ctypes.c_longlong, _vp, ctypes.c_longlong, _vp,
                                       ctypes.c_longlong, _i]),
        "hbem_arnoldi_sv_batch": (_i, [_i, _i, _u, _i, _d, _dp, _dp, _ip]),
        "hbem_arnoldi_sv_batch_device": (_i, [_i, _i, _u, _i, _d, _vp, ctypes.c_longlong, ctypes.c_longlong, _dp, _ip,
                                              _ip]),
        "hbem_cgemm_f32_batch_device": (_i, [_i, _i, _i, _vp, ctypes.c_longlong, ctypes.c_longlong, _vp,
                                             ctypes.c_longlong, ctypes.c_longlong, _vp, ctypes.c_longlong,
                                             ctypes.c_longlong, _i, _i]),
        "hbem_solop_info": (_i, [_vp, _ip]),
        "hbem_sigma_rsvd_sweep": (_i, [_vp, _dp, _i, _d, _d, _i, _i, _i, ctypes.c_ulonglong, _dp]),
        "hbem_opt_subdiv": (_i, [FN_BATCH, _vp, _d, _d, _i, _i, _d, ctypes.c_ulonglong, _dp, _dp, _i, _ip, _ip, _i,
                                 _ip]),
        "hbem_find_resonances_adaptive": (_i, [_vp, _d, _d, _d, _d, _i, _i, _d, _d, ctypes.c_ulonglong, _i, _i, _dp, _i,
                                               _ip, _ip, _ip]),
        "hbem_lu_factor_batch_device": (_i, [_i, _i, _vp, ctypes.c_longlong, _vp, _ip]),
        "hbem_lu_factor_batch_device_f32": (_i, [_i, _i, _vp, ctypes.c_longlong, _vp, _ip]),
        "hbem_lu_solve_batch_device": (_i, [_i, _i, _i, _vp, ctypes.c_longlong, _vp, _i, _vp, ctypes.c_longlong]),
        "hbem_find_resonances_plain": (_i, [_vp, _d, _d, _i, _d, _d, _d, _dp, _i, _ip, _dp, _ip]),
        "hbem_find_resonances_plain_verified": (_i, [_vp, _d, _d, _i, _d, _d, _d, _dp, _i, _ip, _dp, _ip, _dp]),
        "hbem_rtsafe": (_d, [FN, FN_BOTH, _vp, _d, _d, _d, _ip, _up]),
        "hbem_zbrent": (_d, [FN, _vp, _d, _d, _d, _ip, _up]),
        "hbem_brent_min": (_d, [FN, _vp, _d, _d, _d]),
        "hbem_brent_rc_create": (_i, [_d, _d, _d, ctypes.POINTER(_vp)]),
        "hbem_brent_rc_step": (_d, [_vp, _ip, _d]),
        "hbem_brent_rc_destroy": (_i, [_vp]),
        "hbem_brent_guess": (_d, [FN, _vp, _d, _d, _d, _d, _d, _up]),
        "hbem_brent_gsl": (_d, [FN, _vp, _d, _d, _d, _d, _up]),
        "hbem_brent_gsl_with_values": (_d, [FN, _vp, _d, _d, _d, _d, _d, _d, _d, _up]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def lib():
    global _lib
    if _lib is None:
        _lib = load()
    return _lib


def check(status):
    if status != HBEM_OK:
        raise HbemError(status, lib().hbem_last_error().decode(errors="replace"))


def dptr(a):
    return a.ctypes.data_as(_dp)


def iptr(a):
    return a.ctypes.data_as(_ip)
