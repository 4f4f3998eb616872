"""ctypes binding of libthesis_lbm.so (include/thesis_lbm.h).

The library is required: there is no CPU fallback.  If it has not been built,
every call raises with the command that builds it.
"""
import ctypes as C
import os

from . import build as _build

LBM_OK, LBM_DIVERGED, LBM_ERR_FILE, LBM_ERR_UNSUPPORTED, LBM_ERR_INVALID, LBM_ERR_CUDA, LBM_ERR_NOMEM = range(7)
STORE_F32, STORE_F16S, STORE_F64, STORE_F16C = 0, 1, 2, 3
MODE_REFERENCE, MODE_PHYSICS = 0, 1
BGKW, TRT, MRT = 1, 2, 3
INLET, NO_INLET, INLET_PRESSURE = 1, 2, 4
OUTLET_ZOUHE, OUTLET_SECOND, OUTLET_FIRST, OUTLET_HEMODEL, OUTLET_PRESSURE = 1, 2, 3, 4, 5
CURVED, STRAIGHT = 1, 2
WALL_SIMPLE, WALL_COMPLEX = 1, 2
BC_WALL, BC_INLET, BC_OUTLET, BC_PERIODIC, BC_SYMMETRY = 1, 2, 3, 4, 5
NORMS = 5

_IP = C.POINTER(C.c_int)


class LatticeDesc(C.Structure):
    _fields_ = [("dims", C.c_int), ("n", C.c_int), ("m", C.c_int), ("h", C.c_int),
                ("node_type", _IP), ("num_conns", C.c_int),
                ("bc_i", _IP), ("bc_j", _IP), ("bc_k", _IP),
                ("bc_dir", _IP), ("bc_type", _IP), ("bc_id", _IP)]


class Params(C.Structure):
    _fields_ = [("u", C.c_double), ("v", C.c_double), ("w", C.c_double), ("rho", C.c_double),
                ("viscosity", C.c_double), ("g", C.c_double),
                ("inlet_profile", C.c_int), ("outlet_profile", C.c_int),
                ("collision_model", C.c_int), ("boundary_type", C.c_int),
                ("bc_wall_model", C.c_int), ("update_inlet_outlet", C.c_int),
                ("mode", C.c_int), ("storage", C.c_int),
                ("rho_in", C.c_double), ("rho_out", C.c_double), ("f16_scale", C.c_double),
                ("periodic", C.c_int * 3), ("init_equilibrium", C.c_int)]


class CgParams(C.Structure):
    _fields_ = [("r_alpha", C.c_double), ("b_alpha", C.c_double),
                ("r_viscosity", C.c_double), ("b_viscosity", C.c_double),
                ("beta", C.c_double), ("A", C.c_double), ("g_limit", C.c_double),
                ("control_param", C.c_double), ("high_order", C.c_int), ("enhanced", C.c_int),
                ("storage", C.c_int)]


class RunConfig(C.Structure):
    """lbm_run_config (include/thesis_lbm_io.h)."""
    _fields_ = [("problem_name", C.c_char * 512),
                ("u", C.c_double), ("v", C.c_double), ("w", C.c_double), ("rho", C.c_double),
                ("viscosity", C.c_double),
                ("inlet_profile", C.c_int), ("collision_model", C.c_int), ("boundary_type", C.c_int),
                ("bc_wall_model", C.c_int), ("outlet_profile", C.c_int), ("iterations", C.c_int),
                ("autosave_after", C.c_int), ("autosave_every", C.c_int),
                ("stop_condition", C.c_double * 4), ("output_format", C.c_int),
                ("use_initial_conditions_file", C.c_int), ("initial_conditions_name", C.c_char * 512),
                ("residual_model", C.c_int), ("show_macro_diff", C.c_int), ("g", C.c_double),
                ("boundary_id", C.c_int), ("update_inlet_outlet", C.c_int), ("unparsed_lines", C.c_int)]


class UnetConfig(C.Structure):
    """lbm_unet_config (include/thesis_unet.h)."""
    _fields_ = [("height", C.c_int), ("width", C.c_int), ("in_channels", C.c_int), ("out_channels", C.c_int),
                ("max_batch", C.c_int), ("seed", C.c_ulonglong), ("levels", C.c_int),
                ("base_channels", C.c_int), ("max_channels", C.c_int)]


_lib = None


def library_path():
    return _build.LIB_PATH


def lib():
    """Load the native library (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError("libthesis_lbm.so is not built (%s); run "
                           "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    L = C.CDLL(path)
    vp = C.c_void_p
    fp = C.POINTER(C.c_float)
    dp = C.POINTER(C.c_double)
    sig = {
        "lbm_version": (C.c_int, []),
        "lbm_last_error": (C.c_char_p, []),
        "lbm_create": (C.c_int, [C.POINTER(LatticeDesc), C.POINTER(Params), C.POINTER(vp)]),
        "lbm_set_inlet_velocity": (C.c_int, [vp, fp, fp, fp]),
        "lbm_set_link_q": (C.c_int, [vp, dp]),
        "lbm_reference_drag_lift": (C.c_int, [vp, C.c_int, fp, fp, dp]),
        "lbm_link_q": (C.c_int, [C.c_int] * 5 + [_IP] * 4 + [fp] * 6 + [C.c_double, dp]),
        "lbm_init": (C.c_int, [vp, fp, fp, fp, fp]),
        "lbm_step": (C.c_int, [vp, C.c_int, C.c_int, vp]),
        "lbm_get_macro": (C.c_int, [vp, fp, fp, fp, fp]),
        "lbm_get_populations": (C.c_int, [vp, dp]),
        "lbm_set_populations": (C.c_int, [vp, dp]),
        "lbm_state_bytes": (C.c_longlong, [vp]),
        "lbm_get_state": (C.c_int, [vp, vp]),
        "lbm_set_state": (C.c_int, [vp, vp]),
        "lbm_macro_norms": (C.c_int, [vp, dp]),
        "lbm_status": (C.c_int, [vp]),
        "lbm_fluid_nodes": (C.c_longlong, [vp]),
        "lbm_bytes_per_update": (C.c_int, [vp]),
        "lbm_kernel_variant": (C.c_int, [vp]),
        "lbm_kernel_warning": (C.c_char_p, [vp]),
        "lbm_jit_check": (C.c_int, [C.c_int] * 11),
        "lbm_autotune": (C.c_int, [vp, C.c_int, _IP, _IP, _IP]),
        "lbm_kernel_config": (C.c_int, [vp, _IP, _IP, _IP]),
        "lbm_destroy": (None, [vp]),
        "lbm_build_flags": (C.c_int, [C.POINTER(LatticeDesc), C.POINTER(Params),
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_int32), C.POINTER(C.c_int)]),
        "lbm_macro_diff": (C.c_int, [vp, dp]),
        "lbm_residual_l2": (C.c_int, [vp, dp]),
        "lbm_residual_fd_rel_diff": (C.c_int, [vp, dp]),
        "lbm_momentum_exchange": (C.c_int, [vp, _IP, dp]),
        "lbm_read_init_file": (C.c_int, [C.c_char_p, C.POINTER(RunConfig)]),
        "lbm_count_lines": (C.c_longlong, [C.c_char_p]),
        "lbm_pack_spheres": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.c_ulonglong, C.c_int, C.c_double, C.c_longlong, vp, vp, C.c_longlong,
                                       C.POINTER(C.c_longlong)]),
        "lbm_emit_sphere_duct": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                           C.c_ulonglong, C.c_char_p, C.c_char_p, C.POINTER(C.c_longlong)]),
        "lbm_emit_channel2d": (C.c_int, [C.c_int, C.c_int, C.c_ulonglong, C.c_int, C.c_double, C.c_char_p,
                                         C.c_char_p]),
        "lbm_emit_cavity": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_char_p]),
        "lbm_emit_last_error": (C.c_char_p, []),
        "lbm_node_file_dims": (C.c_int, [C.c_char_p]),
        "lbm_read_node_file": (C.c_int, [C.c_char_p, C.c_int, C.c_longlong, _IP, _IP, _IP, fp, fp, fp, _IP]),
        "lbm_read_bc_file": (C.c_int, [C.c_char_p, C.c_int, C.c_longlong, _IP, _IP, _IP, _IP, _IP, fp, fp, fp,
                                       _IP]),
        "lbm_write_results": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, fp, fp, fp, fp, fp, fp,
                                        fp]),
        "lbm_read_results": (C.c_longlong, [C.c_char_p, C.c_longlong, dp]),
        "lbm_read_initial_conditions": (C.c_int, [C.c_char_p, C.c_longlong, C.c_int, C.c_int, C.c_int, fp, fp, fp,
                                                  fp]),
        "lbm_compare_results": (C.c_int, [C.c_char_p, C.c_char_p, dp, dp]),
        "lbm_write_midlines": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, fp, fp, fp, fp, fp, fp,
                                         C.c_double]),
        "lbm_write_cross_section": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, fp, fp, fp, fp, fp, fp,
                                              C.c_double]),
        "lbm_io_last_error": (C.c_char_p, []),
        "lbm_cg_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(CgParams), C.POINTER(vp)]),
        "lbm_cg_create3d": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(CgParams), C.POINTER(vp)]),
        "lbm_cg_get_macro3d": (C.c_int, [vp, fp, fp, fp, fp, fp]),
        "lbm_cg_q": (C.c_int, [vp]),
        "lbm_cg_init": (C.c_int, [vp, fp, fp]),
        "lbm_cg_step": (C.c_int, [vp, C.c_int, C.c_int, vp]),
        "lbm_cg_get_macro": (C.c_int, [vp, fp, fp, fp, fp]),
        "lbm_cg_get_populations": (C.c_int, [vp, fp, fp]),
        "lbm_cg_laplace": (C.c_int, [vp, dp]),
        "lbm_cg_nodes": (C.c_longlong, [vp]),
        "lbm_cg_last_error": (C.c_char_p, []),
        "lbm_cg_destroy": (None, [vp]),
        "lbm_unet_create": (C.c_int, [C.POINTER(UnetConfig), C.POINTER(vp)]),
        "lbm_unet_param_count": (C.c_longlong, [vp]),
        "lbm_unet_get_params": (C.c_int, [vp, fp]),
        "lbm_unet_set_params": (C.c_int, [vp, fp]),
        "lbm_unet_set_dataset": (C.c_int, [vp, C.c_int, fp, fp, fp]),
        "lbm_unet_train_step": (C.c_int, [vp, C.c_int, _IP, C.c_float, dp]),
        "lbm_unet_gradients": (C.c_int, [vp, C.c_int, _IP, fp, dp]),
        "lbm_unet_predict": (C.c_int, [vp, C.c_int, fp, fp]),
        "lbm_unet_last_ms": (C.c_double, [vp]),
        "lbm_unet_last_error": (C.c_char_p, []),
        "lbm_unet_destroy": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class LbmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("lbm error %d: %s" % (code, msg))
        self.code = code


def check(rc):
    if rc != LBM_OK:
        raise LbmError(rc, lib().lbm_last_error().decode(errors="replace"))
    return rc


def check_cg(rc):
    if rc != LBM_OK:
        raise LbmError(rc, lib().lbm_cg_last_error().decode(errors="replace"))
    return rc


def check_unet(rc):
    if rc != LBM_OK:
        raise LbmError(rc, lib().lbm_unet_last_error().decode(errors="replace"))
    return rc
