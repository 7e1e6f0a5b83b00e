"""ctypes binding of the C ABI (include/panslbm_gb300.h).

The shared library is built in-tree by panslbm2_gb300/build.py. Loading fails loudly when it
is missing: there is no CPU fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpanslbm_gb300.so")

PL_OK = 0
PL_ERR_ARG, PL_ERR_CUDA, PL_ERR_UNSUPPORTED, PL_ERR_STATE, PL_ERR_ALLOC, PL_ERR_NONFINITE = -1, -2, -3, -4, -5, -6
PL_CONVERGED, PL_MAX_STEPS, PL_DIVERGED = 1, 2, 3
PL_FP64, PL_FP32, PL_FP16, PL_BF16 = 0, 1, 2, 3
STORAGE = {"fp64": PL_FP64, "fp32": PL_FP32, "fp16": PL_FP16, "bf16": PL_BF16}

# collide kinds
NS_COLLIDE, NS_BRINKMAN, AD_NATURAL, AD_FORCE, AD_HEATEX, AD_NATURAL_NOBRINK, AD_FORCE_NOBRINK = 0, 1, 2, 3, 4, 5, 6
NSIN_COLLIDE, NSIN_BRINKMAN = 7, 8
ANS_BRINKMAN, AAD_NATURAL, AAD_FORCE, AAD_HEATEX, AAD_MASSFLOW, ANSIN_BRINKMAN = 10, 11, 12, 13, 14, 15
EL_COLLIDE, EL_EXTENDED, AEL_COLLIDE = 16, 17, 18
# boundary op kinds
BC_WALL, BC_IWALL, BC_NS_U, BC_NS_RHO, BC_AD_T, BC_AD_Q, BC_AD_QC = 0, 1, 2, 3, 4, 5, 6
BC_ANS_U, BC_ANS_RHO, BC_AAD_T, BC_AAD_Q, BC_AAD_RHO = 7, 8, 9, 10, 11
BC_NSIN_U, BC_NSIN_RHO, BC_ANSIN_U = 12, 13, 14
BC_EL_STRESS, BC_AEL_STRESS = 15, 16
SMOOTH_CORNER, SMOOTH_AT, SMOOTH_LINE = 20, 21, 22
# fields
ALPHA, KAPPA, BETA, DIRX, DIRY, DIRZ, DENSITY, GAMMA = 0, 1, 2, 3, 4, 5, 6, 7
OPT_GRAPHS, OPT_SIDE_PRIORITY, OPT_STOCHASTIC_ROUNDING, OPT_SNAPSHOT_IN_STEP = 1, 2, 3, 4
RHO, UX, UY, UZ, TEM, QX, QY, QZ = 8, 9, 10, 11, 12, 13, 14, 15
IP, IUX, IUY, IUZ, IMX, IMY, IMZ, ITEM, IQX, IQY, IQZ = 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26
FWD_RHO, FWD_UX, FWD_UY, FWD_UZ, FWD_TEM = 32, 33, 34, 35, 36
DFDS, DADS, DKDS, QN, ACC = 37, 38, 39, 40, 41
HEAT_SOURCE, OBJ_WEIGHT = 42, 43
STORE_POPS, STORE_FWD, STORE_SNAP = 0, 1, 2
# the elastic kinds' macros share the planes above
SXX, SXY, SYX, SYY = TEM, QX, QY, QZ
IRHO, ISXX, ISXY, ISYX, ISYY = IP, ITEM, IQX, IQY, IQZ

DP = C.POINTER(C.c_double)
IPT = C.POINTER(C.c_int)


class Phys(C.Structure):
    _fields_ = [("nu", C.c_double), ("diff", C.c_double), ("gx", C.c_double), ("gy", C.c_double),
                ("gz", C.c_double), ("tem0", C.c_double), ("tau", C.c_double)]


class BcDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("lat", C.c_int), ("axis", C.c_int), ("pos", C.c_int), ("dir", C.c_int),
                ("type", IPT), ("v0", DP), ("v1", DP), ("v2", DP), ("c0", C.c_double), ("c1", C.c_double),
                ("c2", C.c_double), ("eps", C.c_double), ("kappa", C.c_double), ("i", C.c_int), ("j", C.c_int),
                ("k", C.c_int), ("di", C.c_int), ("dj", C.c_int), ("dk", C.c_int)]


EXPORTS = [
    "pl_create", "pl_destroy", "pl_last_error", "pl_synchronize", "pl_set_stream", "pl_set_option",
    "pl_set_shift", "pl_set_inflow_scale",
    "pl_set_populations", "pl_get_populations", "pl_set_field", "pl_get_field", "pl_get_saved_field", "pl_freeze_forward",
    "pl_program_create", "pl_program_destroy", "pl_init", "pl_init_elastic", "pl_collide", "pl_step", "pl_steps", "pl_stream",
    "pl_solve", "pl_snapshot", "pl_set_snapshot", "pl_residual", "pl_residual_host", "pl_residual_device_noalloc",
    "pl_sensitivity", "pl_sensitivity_compliance", "pl_store", "pl_load", "pl_store_release", "pl_store_swap_snapshot",
    "pl_sensitivity_device", "pl_accumulate", "pl_heaviside_var",
    "pl_heaviside_sens", "pl_density_filter", "pl_filter_taps", "pl_filter_weighted", "pl_normalize", "pl_stats", "pl_mma_create", "pl_mma_set_param",
    "pl_mma_update", "pl_mma_destroy", "pl_mma_get_state", "pl_mma_set_state", "pl_debug_fail_alloc",
    "pl_unet_create", "pl_unet_destroy", "pl_unet_param_count", "pl_unet_init_params", "pl_unet_get_params",
    "pl_unet_set_params", "pl_unet_forward", "pl_unet_backward", "pl_unet_gradients", "pl_unet_dataset_reserve",
    "pl_unet_set_static", "pl_unet_add_sample", "pl_unet_add_sample_lattice", "pl_unet_train", "pl_unet_set_norm", "pl_unet_get_norm",
    "pl_unet_predict", "pl_probe_fp64_fma",
]

_lib = None


class PanslbmError(RuntimeError):
    pass


def load():
    """Load the CUDA library (built by build.py); raise if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise PanslbmError("CUDA library %s is not built (run panslbm2_gb300/build.py); "
                           "there is no CPU fallback" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    lib.pl_last_error.restype = C.c_char_p
    for name in EXPORTS:
        fn = getattr(lib, name)
        if name != "pl_last_error":
            fn.restype = C.c_int
    _lib = lib
    return lib


def check(code):
    if code != PL_OK:
        msg = _lib.pl_last_error().decode() if _lib is not None else ""
        raise PanslbmError("panslbm_gb300 error %d: %s" % (code, msg))
    return code
