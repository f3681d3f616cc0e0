"""ctypes binding of the C ABI declared in include/maestro_adv.h (libmaestro_adv.so).

The shared library is built in-tree by ``maestroex_gb300.build.build_library()``; importing
this module never falls back to anything else: if the library is missing the load fails
loudly.
"""
import ctypes as C
import os

from .params import MadvParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmaestro_adv.so")

MADV_OK = 0
MODE_BATCHED, MODE_PER_BOX, MODE_GRAPH = 0, 1, 2

ERRORS = {
    -1: "MADV_ERR_PARAM", -2: "MADV_ERR_LAYOUT", -3: "MADV_ERR_UNSUPPORTED",
    -4: "MADV_ERR_CUDA", -5: "MADV_ERR_STATE", -6: "MADV_ERR_EOS", -7: "MADV_ERR_NOCONV",
}

EXPORTED = [
    "madv_ctx_create", "madv_ctx_destroy", "madv_set_dt", "madv_set_layout",
    "madv_set_base_state", "madv_advance_premac", "madv_addw0", "madv_density_advance",
    "madv_enthalpy_advance", "madv_stage_forward", "madv_last_launch_count",
    "madv_last_error", "madv_version", "madv_profile", "madv_profile_report", "madv_probe_fp64_peak",
    "madv_selftest_exact", "madv_ppm", "madv_ppm_noalloc", "madv_set_layout_levels",
    "madv_set_base_state_levels", "madv_stage_forward_levels", "madv_stage_adjoint",
    "madv_autotune_trial", "madv_autotune_ppm_trial", "madv_autotune_finish", "madv_autotune_apply",
    "madv_make_utrans", "madv_vel_pred", "madv_make_edge_scal", "madv_make_rhox_flux", "madv_make_rhoh_flux",
    "madv_update_scal", "madv_velocity_advance", "madv_est_dt", "madv_mac_project", "madv_mac_project_levels",
    "madv_set_option",
]


class MadvDtParams(C.Structure):
    _fields_ = [("cfl", C.c_double), ("drdxfac", C.c_int), ("max_dt", C.c_double), ("fixed_dt", C.c_double),
                ("small_dt", C.c_double)]


class MadvDtResult(C.Structure):
    _fields_ = [("dt", C.c_double), ("dt_estimate", C.c_double), ("umax", C.c_double), ("rel_eps", C.c_double)]


class MadvMacResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("resid_ratio", C.c_double)]


class MadvBox(C.Structure):
    _fields_ = [("lo", C.c_int * 3), ("hi", C.c_int * 3)]


class MadvFab(C.Structure):
    _fields_ = [("p", C.c_void_p), ("lo", C.c_int * 3), ("hi", C.c_int * 3), ("ncomp", C.c_int)]


class MadvMultiFab(C.Structure):
    _fields_ = [("nfab", C.c_int), ("fab", C.POINTER(MadvFab))]


class MadvBaseState(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in (
        "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new", "p0_old", "p0_new", "psi", "grav_cell",
        "w0_force", "w0", "rho0_predicted_edge")]


class MadvAdjSeed(C.Structure):
    _fields_ = [("nsteps", C.c_int), ("ckpt_interval", C.c_int), ("uold", C.POINTER(MadvMultiFab)),
                ("sold0", C.POINTER(MadvMultiFab)), ("weight", C.POINTER(MadvMultiFab))]


class MadvAdjResult(C.Structure):
    _fields_ = [("sfinal", C.POINTER(MadvMultiFab)), ("grad_s", C.POINTER(MadvMultiFab)),
                ("grad_u", C.POINTER(MadvMultiFab)), ("J", C.c_double), ("device_bytes", C.c_longlong)]


class MadvError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is missing: run maestroex_gb300.build.build_library() first")
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.madv_ctx_create.argtypes = [P(MadvParams), P(C.c_void_p)]
        L.madv_ctx_destroy.argtypes = [C.c_void_p]
        L.madv_ctx_destroy.restype = None
        L.madv_set_dt.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.madv_set_layout.argtypes = [C.c_void_p, C.c_int, P(MadvBox)]
        L.madv_set_base_state.argtypes = [C.c_void_p, P(MadvBaseState)]
        L.madv_set_layout_levels.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(MadvBox)]
        L.madv_set_base_state_levels.argtypes = [C.c_void_p, C.c_int, P(MadvBaseState)]
        MF = P(MadvMultiFab)
        L.madv_advance_premac.argtypes = [C.c_void_p, MF, MF, MF, MF, MF, C.c_void_p]
        L.madv_addw0.argtypes = [C.c_void_p, MF, C.c_double, C.c_void_p]
        L.madv_density_advance.argtypes = [C.c_void_p, C.c_int, MF, MF, MF, MF, MF, MF, C.c_void_p]
        L.madv_enthalpy_advance.argtypes = [C.c_void_p, C.c_int, MF, MF, MF, MF, MF, MF, C.c_void_p]
        I = C.c_int
        L.madv_make_utrans.argtypes = [C.c_void_p, MF, MF, MF, C.c_void_p]
        L.madv_vel_pred.argtypes = [C.c_void_p, MF, MF, MF, MF, MF, C.c_void_p]
        L.madv_make_edge_scal.argtypes = [C.c_void_p, MF, MF, MF, MF, I, I, I, I, I, C.c_void_p]
        L.madv_make_rhox_flux.argtypes = [C.c_void_p, I, MF, MF, MF, MF, I, I, C.c_void_p]
        L.madv_make_rhoh_flux.argtypes = [C.c_void_p, I, MF, MF, MF, C.c_void_p]
        L.madv_update_scal.argtypes = [C.c_void_p, MF, MF, MF, MF, I, I, C.c_void_p]
        L.madv_velocity_advance.argtypes = [C.c_void_p, MF, MF, MF, MF, MF, MF, MF, MF, C.c_void_p]
        L.madv_est_dt.argtypes = [C.c_void_p, I, MF, MF, MF, P(MadvDtParams), P(MadvDtResult), C.c_void_p]
        L.madv_mac_project.argtypes = [C.c_void_p, MF, MF, MF, MF, P(C.c_double), C.c_double, I, P(MadvMacResult),
                                       C.c_void_p]
        L.madv_mac_project_levels.argtypes = [C.c_void_p, I, MF, MF, MF, MF, P(C.c_double), C.c_double, I,
                                              P(MadvMacResult), C.c_void_p]
        L.madv_stage_forward.argtypes = [C.c_void_p, C.c_int, MF, MF, MF, MF, MF, MF, MF, MF, MF,
                                         C.c_void_p]
        L.madv_stage_forward_levels.argtypes = [C.c_void_p, C.c_int, C.c_int, MF, MF, MF, MF, MF, MF, MF, MF, MF,
                                                C.c_void_p]
        L.madv_stage_adjoint.argtypes = [C.c_void_p, P(MadvAdjSeed), P(MadvAdjResult), C.c_void_p]
        L.madv_autotune_trial.argtypes = [C.c_void_p, C.c_int]
        L.madv_autotune_ppm_trial.argtypes = [C.c_void_p, C.c_int]
        L.madv_autotune_finish.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
        L.madv_autotune_apply.argtypes = [C.c_void_p, C.c_char_p]
        FAB = P(MadvFab)
        L.madv_ppm.argtypes = [C.c_void_p, P(MadvBox), FAB, C.c_int, FAB, FAB, FAB, C.c_int, P(C.c_int), FAB, FAB,
                               C.c_void_p]
        L.madv_ppm_noalloc.argtypes = [P(MadvParams), P(MadvBox), FAB, C.c_int, FAB, FAB, FAB, C.c_int, P(C.c_int),
                                       FAB, FAB, C.c_void_p]
        L.madv_last_launch_count.argtypes = [C.c_void_p]
        L.madv_last_launch_count.restype = C.c_long
        L.madv_profile.argtypes = [C.c_void_p, C.c_int]
        L.madv_set_option.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
        L.madv_profile_report.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
        L.madv_probe_fp64_peak.argtypes = [P(C.c_double), C.c_void_p]
        L.madv_selftest_exact.argtypes = [C.c_double, C.c_double, C.c_longlong, P(C.c_longlong), C.c_void_p]
        L.madv_last_error.restype = C.c_char_p
        L.madv_version.restype = C.c_char_p
        _lib = L
    return _lib


def check(rc):
    if rc != MADV_OK:
        raise MadvError(rc, lib().madv_last_error().decode())
    return rc
