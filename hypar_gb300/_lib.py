"""ctypes binding of libgbhypar's C ABI (include/gbhypar.h).

The library is loaded from this package's directory; there is no fallback:
if libgbhypar.so is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbhypar.so")

GB_OK = 0
GB_ERR = {1: "GB_ERR_ARG", 2: "GB_ERR_CUDA", 3: "GB_ERR_INPUT", 4: "GB_ERR_UNSUPPORTED", 5: "GB_ERR_NOMEM",
          6: "GB_ERR_NONFINITE", 7: "GB_ERR_HOOK"}
MODEL = {"euler1d": 1, "euler2d": 2, "navierstokes3d": 3}
UPWIND = {"roe": 0, "llf-char": 1, "rf-char": 2, "rusanov": 3, "steger-warming": 4}
INTERP = {"components": 0, "characteristic": 1}
WENO_WEIGHTS = {"js": 0, "mapped": 1, "borges": 2, "yc": 3, "none": 4}
SCHEME = {"weno5": 0, "crweno5": 1}
LAYOUT_INTERIOR, LAYOUT_GHOSTED = 0, 1
MEM_HOST, MEM_DEVICE = 0, 1

# Every symbol include/gbhypar.h declares.
EXPORTS = [
    "gb_last_error", "gb_inputs_read", "gb_inputs_free", "gb_inputs_config", "gb_inputs_x", "gb_inputs_dxinv",
    "gb_inputs_u0", "gb_rk_table", "gb_solver_create", "gb_solver_destroy", "gb_solver_config",
    "gb_solver_set_stream", "gb_solver_sync", "gb_solver_set_state", "gb_solver_get_state", "gb_solver_state",
    "gb_solver_step", "gb_solver_time", "gb_solver_set_launch", "gb_solver_check_finite", "gb_run_case",
    "gb_write_binary", "gb_write_text", "gb_write_tecplot", "gb_diff_binary", "gb_HyperbolicFunction", "gb_ParabolicFunction", "gb_SourceFunction", "gb_FFunction",
    "gb_GFunction", "gb_UFunction", "gb_Upwind", "gb_SetInterpLimiterVar", "gb_InterpolateInterfacesHyp", "gb_ApplyBoundaryConditions", "gb_RHSFunctionExplicit",
    "gb_TimeRK", "gb_probe_fp64_peak", "gb_probe_rcp_sqrt", "gb_solver_profile", "gb_solver_profile_read",
    "gb_solver_get_launch", "gb_solver_autotune", "gb_inputs_nsims", "gb_inputs_read_member",
    "gb_ensemble_create", "gb_ensemble_destroy", "gb_ensemble_size", "gb_ensemble_set_stream", "gb_ensemble_sync",
    "gb_ensemble_set_state", "gb_ensemble_get_state", "gb_ensemble_step", "gb_ensemble_time",
    "gb_ensemble_set_launch", "gb_ensemble_get_launch", "gb_ensemble_autotune", "gb_rhs_explicit_noalloc",
    "gb_adjoint_create", "gb_adjoint_create_ex", "gb_adjoint_destroy", "gb_adjoint_set_stream", "gb_adjoint_sync", "gb_adjoint_set_launch",
    "gb_adjoint_get_launch", "gb_adjoint_info", "gb_adjoint_rhs_vjp", "gb_adjoint_rhs_jvp", "gb_adjoint_forward",
    "gb_adjoint_backward", "gb_adjoint_tlm", "gb_inputs_exact", "gb_solver_set_time", "gb_solver_cfl",
    "gb_solver_step_report", "gb_solver_error", "gb_op_to_initial", "gb_inputs_gravity_field",
    "gb_solver_set_gravity_field", "gb_solver_conservation_begin", "gb_solver_conservation_error",
    "gb_ensemble_conservation_begin", "gb_ensemble_conservation_error", "gb_ensemble_error",
    "gb_solver_set_hooks", "gb_inputs_zone_temperature", "gb_solver_set_zone_temperature",
    "gb_inputs_zone_sponge", "gb_solver_set_zone_sponge", "gb_inputs_zone_inflow", "gb_solver_set_zone_inflow",
]


class GbConfig(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int), ("ndims", ctypes.c_int), ("nvars", ctypes.c_int), ("ghosts", ctypes.c_int),
        ("dim", ctypes.c_int * 3), ("interp", ctypes.c_int), ("upwind", ctypes.c_int),
        ("gamma", ctypes.c_double), ("weno_eps", ctypes.c_double),
        ("Re", ctypes.c_double), ("Pr", ctypes.c_double), ("Minf", ctypes.c_double),
        ("nzones", ctypes.c_int), ("zones", (ctypes.c_int * 9) * 12),
        ("rk_nstages", ctypes.c_int), ("rk_A", ctypes.c_double * 16), ("rk_b", ctypes.c_double * 4),
        ("rk_c", ctypes.c_double * 4), ("dt", ctypes.c_double), ("n_iter", ctypes.c_int),
        ("file_op_iter", ctypes.c_int), ("weno_weights", ctypes.c_int), ("restart_iter", ctypes.c_int),
        ("screen_op_iter", ctypes.c_int), ("write_residual", ctypes.c_int),
        ("zone_data", (ctypes.c_double * 8) * 12),
        ("gravity", ctypes.c_double * 3), ("rho_ref", ctypes.c_double), ("p_ref", ctypes.c_double),
        ("R_gas", ctypes.c_double), ("N_bv", ctypes.c_double), ("HB", ctypes.c_int), ("hyp_scheme", ctypes.c_int),
        ("grav_type", ctypes.c_int), ("cons_check", ctypes.c_int), ("par_scheme", ctypes.c_int),
    ]


class GbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{GB_ERR.get(code, code)}: {msg}")
        self.code = code


_lib = None

VP = ctypes.c_void_p
DP = ctypes.POINTER(ctypes.c_double)
FFUNC = ctypes.CFUNCTYPE(ctypes.c_int, DP, DP, ctypes.c_int, VP, ctypes.c_double)
# HyPar's stage / step hooks (include/hypar.h:334-341)
PRESTAGE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.POINTER(DP), VP, VP, ctypes.c_double)
POSTSTAGE = ctypes.CFUNCTYPE(ctypes.c_int, VP, VP, VP, ctypes.c_double)
PRESTEP = ctypes.CFUNCTYPE(ctypes.c_int, VP, VP, VP, ctypes.c_double)
POSTSTEP = ctypes.CFUNCTYPE(ctypes.c_int, VP, VP, VP, ctypes.c_double, ctypes.c_int)
UPWFUNC = ctypes.CFUNCTYPE(ctypes.c_int, DP, DP, DP, DP, DP, DP, ctypes.c_int, VP, ctypes.c_double)


def lib():
    """Load libgbhypar.so (raises if it is absent: there is no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with hypar_gb300.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    L.gb_last_error.restype = ctypes.c_char_p
    L.gb_inputs_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(VP)]
    L.gb_inputs_free.argtypes = [VP]
    L.gb_inputs_free.restype = None
    L.gb_inputs_config.argtypes = [VP]
    L.gb_inputs_config.restype = ctypes.POINTER(GbConfig)
    for n in ("gb_inputs_x", "gb_inputs_dxinv", "gb_inputs_u0", "gb_inputs_exact", "gb_inputs_gravity_field"):
        getattr(L, n).argtypes = [VP]
        getattr(L, n).restype = DP
    L.gb_rk_table.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), DP, DP, DP]
    L.gb_solver_create.argtypes = [ctypes.POINTER(GbConfig), DP, ctypes.c_int, ctypes.POINTER(VP)]
    L.gb_solver_destroy.argtypes = [VP]
    L.gb_solver_destroy.restype = None
    L.gb_solver_config.argtypes = [VP]
    L.gb_solver_config.restype = ctypes.POINTER(GbConfig)
    L.gb_solver_set_stream.argtypes = [VP, VP]
    L.gb_solver_sync.argtypes = [VP]
    L.gb_solver_set_state.argtypes = [VP, VP, ctypes.c_int, ctypes.c_int]
    L.gb_solver_get_state.argtypes = [VP, VP, ctypes.c_int, ctypes.c_int]
    L.gb_solver_state.argtypes = [VP]
    L.gb_solver_state.restype = VP
    L.gb_solver_step.argtypes = [VP, ctypes.c_int]
    L.gb_solver_time.argtypes = [VP]
    L.gb_solver_time.restype = ctypes.c_double
    L.gb_solver_set_launch.argtypes = [VP, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.gb_solver_check_finite.argtypes = [VP, ctypes.POINTER(ctypes.c_int)]
    L.gb_run_case.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
    L.gb_write_binary.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), DP, DP]
    L.gb_write_text.argtypes = L.gb_write_binary.argtypes
    L.gb_diff_binary.argtypes = [ctypes.c_char_p, ctypes.c_char_p, DP, DP]
    L.gb_write_tecplot.argtypes = L.gb_write_binary.argtypes
    L.gb_HyperbolicFunction.argtypes = [VP, VP, VP, VP, ctypes.c_double, ctypes.c_int, VP, VP]
    for n in ("gb_ParabolicFunction", "gb_SourceFunction", "gb_RHSFunctionExplicit"):
        getattr(L, n).argtypes = [VP, VP, VP, VP, ctypes.c_double]
    for n in ("gb_FFunction", "gb_GFunction"):
        getattr(L, n).argtypes = [VP, VP, ctypes.c_int, VP, ctypes.c_double]
    L.gb_UFunction.argtypes = [VP, VP, ctypes.c_int, VP, VP, ctypes.c_double]
    L.gb_Upwind.argtypes = [VP, VP, VP, VP, VP, VP, ctypes.c_int, VP, ctypes.c_double]
    L.gb_SetInterpLimiterVar.argtypes = [VP, VP, VP, ctypes.c_int, VP, VP]
    L.gb_InterpolateInterfacesHyp.argtypes = [VP, VP, VP, VP, ctypes.c_int, ctypes.c_int, VP, VP, ctypes.c_int]
    L.gb_ApplyBoundaryConditions.argtypes = [VP, VP, VP, VP, ctypes.c_double]
    L.gb_TimeRK.argtypes = [VP]
    L.gb_solver_set_hooks.argtypes = [VP, PRESTAGE, POSTSTAGE, PRESTEP, POSTSTEP, VP, VP]
    L.gb_probe_fp64_peak.argtypes = [DP]
    L.gb_probe_rcp_sqrt.argtypes = [VP, VP, VP, VP, VP, VP, ctypes.c_longlong]
    L.gb_solver_profile.argtypes = [VP, ctypes.c_int]
    L.gb_solver_get_launch.argtypes = [VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.gb_solver_autotune.argtypes = [VP, ctypes.c_int]
    L.gb_inputs_nsims.argtypes = [ctypes.c_char_p]
    L.gb_inputs_read_member.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(VP)]
    L.gb_ensemble_create.argtypes = [ctypes.POINTER(GbConfig), ctypes.POINTER(DP), ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(VP)]
    L.gb_ensemble_destroy.argtypes = [VP]
    L.gb_ensemble_destroy.restype = None
    L.gb_ensemble_size.argtypes = [VP]
    L.gb_ensemble_set_stream.argtypes = [VP, VP]
    L.gb_ensemble_sync.argtypes = [VP]
    L.gb_ensemble_set_state.argtypes = [VP, ctypes.c_int, VP, ctypes.c_int, ctypes.c_int]
    L.gb_ensemble_get_state.argtypes = [VP, ctypes.c_int, VP, ctypes.c_int, ctypes.c_int]
    L.gb_ensemble_step.argtypes = [VP, ctypes.c_int]
    L.gb_ensemble_time.argtypes = [VP]
    L.gb_ensemble_time.restype = ctypes.c_double
    L.gb_ensemble_set_launch.argtypes = [VP, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.gb_ensemble_get_launch.argtypes = [VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.gb_ensemble_autotune.argtypes = [VP, ctypes.c_int]
    L.gb_solver_profile_read.argtypes = [VP, DP, ctypes.POINTER(ctypes.c_longlong)]
    L.gb_rhs_explicit_noalloc.argtypes = [ctypes.POINTER(GbConfig), VP, VP, VP, VP]
    L.gb_solver_set_time.argtypes = [VP, ctypes.c_double]
    L.gb_solver_set_gravity_field.argtypes = [VP, VP]
    L.gb_inputs_zone_temperature.argtypes = [VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(DP),
                                             ctypes.POINTER(DP)]
    L.gb_solver_set_zone_temperature.argtypes = [VP, ctypes.c_int, ctypes.c_int, DP, DP]
    L.gb_inputs_zone_sponge.argtypes = [VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(DP)]
    L.gb_solver_set_zone_sponge.argtypes = [VP, ctypes.c_int, DP]
    L.gb_inputs_zone_inflow.argtypes = [VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(DP)]
    L.gb_solver_set_zone_inflow.argtypes = [VP, ctypes.c_int, ctypes.c_int, DP]
    L.gb_solver_cfl.argtypes = [VP, DP]
    L.gb_solver_step_report.argtypes = [VP, ctypes.c_int, DP, DP]
    L.gb_solver_error.argtypes = [VP, VP, ctypes.c_int, ctypes.c_int, DP]
    L.gb_solver_conservation_begin.argtypes = [VP]
    L.gb_solver_conservation_error.argtypes = [VP, DP]
    L.gb_ensemble_conservation_begin.argtypes = [VP]
    L.gb_ensemble_conservation_error.argtypes = [VP, ctypes.c_int, DP]
    L.gb_ensemble_error.argtypes = [VP, ctypes.c_int, VP, ctypes.c_int, ctypes.c_int, DP]
    L.gb_op_to_initial.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    L.gb_adjoint_create.argtypes = [ctypes.POINTER(GbConfig), DP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(VP)]
    L.gb_adjoint_create_ex.argtypes = [ctypes.POINTER(GbConfig), DP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_longlong, ctypes.POINTER(VP)]
    L.gb_adjoint_destroy.argtypes = [VP]
    L.gb_adjoint_destroy.restype = None
    L.gb_adjoint_set_stream.argtypes = [VP, VP]
    L.gb_adjoint_sync.argtypes = [VP]
    L.gb_adjoint_set_launch.argtypes = [VP, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.gb_adjoint_get_launch.argtypes = [VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.gb_adjoint_info.argtypes = [VP, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                  ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
    L.gb_adjoint_rhs_vjp.argtypes = [VP, VP, VP, VP]
    L.gb_adjoint_rhs_jvp.argtypes = [VP, VP, VP, VP, VP]
    L.gb_adjoint_forward.argtypes = [VP, VP, VP]
    L.gb_adjoint_backward.argtypes = [VP, VP, VP]
    L.gb_adjoint_tlm.argtypes = [VP, VP, VP, VP, VP]
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != GB_OK:
        raise GbError(rc, lib().gb_last_error().decode(errors="replace"))


def fn_address(name: str) -> int:
    """Address of an exported function (to pass as a HyPar function pointer)."""
    return ctypes.cast(getattr(lib(), name), ctypes.c_void_p).value
