"""ctypes mirror of include/rheocell_gb300.h.

The engine is a C-ABI shared library; this module declares its structs and
function signatures for Python callers (tests, bench, scripts).  Struct layouts
must match the header field for field.
"""
from __future__ import annotations

import ctypes as C

RC_OK = 0
RC_ERR_INVALID = -1
RC_ERR_CUDA = -2
RC_ERR_OOM = -3
RC_ERR_OVERLAP = -4
RC_ERR_NONFINITE = -5
RC_ERR_CG = -6
RC_ERR_CAPACITY = -7
RC_ERR_UNSUPPORTED = -8
RC_NOALLOC_MAX_UNKNOWNS = 32768
RC_NOALLOC_MAX_BOX_SITES = 16384
RC_UNET_PARAMS = 25937
RC_SOLVER_PLAIN = 0
RC_SOLVER_LEARNED = 1
RC_SOLVER_LEARNED_FP32 = 2
RC_SOLVER_PLAIN_FP64 = 3
RC_OBS_VELOCITY = 0
RC_OBS_SHAPE = 1
RC_OBS_NEMATIC = 2
RC_OBS_FORCE = 3
RC_OBS_FORCE_PASSIVE = 4
RC_OBS_FORCE_ACTIVE = 5
RC_OBS_PRESSURE = 6
RC_OBS_THERMO = 7
RC_OBS_THERMO_XY = 8
RC_OBS_CHEMPOT2 = 9
SOLVER_PHASES = ["fcg_setup", "first_layer", "tc_level0", "tc_level1", "tc_level2", "last_layer",
                 "fcg_z", "fcg_direction", "solve_start", "fcg_update", "other",
                 "tc_weights", "tc_staging", "tc_mma", "tc_epilogue",
                 "tc_mma_warp_wait", "tc_mma_warp_issue", "tc_stage_wait", "tc_stage_load"]

RC_SIMPLEFIELD = 0
RC_ACTIVENEMATIC = 1
RC_WETPOLARMODEL = 2
RC_WETMODEL = 3

MODEL_NAMES = {"simplefield": RC_SIMPLEFIELD, "activenematic": RC_ACTIVENEMATIC,
               "wetpolarmodel": RC_WETPOLARMODEL, "wetmodel": RC_WETMODEL}

RC_PRECISION_DOUBLE = 0
RC_PRECISION_MIXED = 1
RC_PRECISION_FLOAT = 2

RC_FIELD_SCALARS = 0x01
RC_FIELD_PHI = 0x02
RC_FIELD_VEL = 0x04
RC_FIELD_MU = 0x08
RC_FIELD_GRAD = 0x10
RC_FIELD_MAP = 0x20
RC_FIELD_ALL = 0x3F

D2 = C.c_double * 2


class RcParams(C.Structure):
    _fields_ = [
        ("model", C.c_int), ("precision", C.c_int), ("R", C.c_int), ("border", C.c_int),
        ("dt", C.c_double), ("J0", C.c_double),
        ("gamma", C.c_double), ("lambda_", C.c_double), ("omega", C.c_double),
        ("mu", C.c_double), ("kappa", C.c_double),
        ("passive_alpha", C.c_double), ("cg_tolerance", C.c_double),
        ("cg_restart_every", C.c_int), ("anchoring", C.c_int),
        ("friction", D2), ("friction_cell", D2), ("zetaQ_self", D2), ("zetaQ_inter", D2),
        ("J_Q", D2), ("beta", D2),
        ("rng_state", C.c_ulonglong), ("rng_has_cached", C.c_int), ("rng_cached", C.c_double),
        ("conserved", C.c_int), ("wall_slip", C.c_double),
    ]


class RcBox(C.Structure):
    _fields_ = [("Lx", C.c_int), ("Ly", C.c_int), ("walls", C.POINTER(C.c_double))]


def make_box(L: int, walls=None) -> RcBox:
    """An rc_box of side L; `walls` (L*L float64 values or None) must stay
    alive until the call that reads the box returns."""
    b = RcBox(L, L)
    if walls is not None:
        b.walls = walls.ctypes.data_as(C.POINTER(C.c_double))
    return b


DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)


class RcCellHost(C.Structure):
    _fields_ = [
        ("lsub_x", C.c_int), ("lsub_y", C.c_int), ("offset_x", C.c_int), ("offset_y", C.c_int),
        ("corner", C.c_int), ("type", C.c_int),
        ("com_x", C.c_double), ("com_y", C.c_double), ("unrap_x", C.c_double), ("unrap_y", C.c_double),
        ("q00", C.c_double), ("q01", C.c_double), ("theta_q", C.c_double), ("theta_q_old", C.c_double),
        ("nemq_x", C.c_double), ("nemq_y", C.c_double), ("nemq_old_x", C.c_double), ("nemq_old_y", C.c_double),
        ("area", C.c_double), ("sum_f", C.c_double), ("perimeter", C.c_double),
        ("s00", C.c_double), ("s01", C.c_double), ("force_rep_x", C.c_double), ("force_rep_y", C.c_double),
        ("capacity", C.c_int),
        ("phi", DP), ("vx", DP), ("vy", DP), ("mu", DP), ("dx", DP), ("dy", DP), ("box_index", IP),
    ]


class RcStepStats(C.Structure):
    _fields_ = [
        ("steps_done", C.c_longlong), ("cg_solves", C.c_int), ("cg_iterations", C.c_int),
        ("cg_max_iterations", C.c_int), ("cg_max_rel_residual", C.c_double),
        ("resized_cells", C.c_int), ("refinements", C.c_int), ("kernel_launches", C.c_longlong),
        ("fallbacks", C.c_int), ("reserved", C.c_int),
    ]


RC_PROFILE_TANH, RC_PROFILE_DISC = 0, 1


class RcGenerateSpec(C.Structure):
    _fields_ = [("profile", C.c_int), ("radius", C.c_double), ("width", C.c_double)]


class RcAutotuneReport(C.Structure):
    _fields_ = [("candidates", C.c_int), ("threads", C.c_int * 4), ("ms_per_step", C.c_double * 4), ("chosen", C.c_int)]


class RcTrainOptions(C.Structure):
    _fields_ = [
        ("epochs", C.c_int), ("batch", C.c_int), ("learning_rate", C.c_double), ("validation", C.c_double),
        ("seed", C.c_ulonglong), ("init", C.c_int), ("max_samples", C.c_int), ("learning_rate_final", C.c_double),
    ]


class RcTrainReport(C.Structure):
    _fields_ = [
        ("samples", C.c_int), ("train_samples", C.c_int), ("validation_samples", C.c_int), ("epochs", C.c_int),
        ("steps", C.c_int), ("loss_first_epoch", C.c_double), ("loss_last_epoch", C.c_double),
        ("validation_loss_init", C.c_double), ("validation_loss", C.c_double), ("ms", C.c_double),
    ]


def declare(lib: C.CDLL, prefix: str) -> C.CDLL:
    """Declare the argument/return types of the rc_*-style API under ``prefix``
    ("rc" for the engine, "orc" for the oracle)."""
    vp = C.c_void_p
    f = lambda name: getattr(lib, "%s_%s" % (prefix, name))
    f("create").argtypes = ([C.POINTER(RcParams), C.POINTER(RcBox), C.c_int, C.POINTER(RcCellHost)]
                            + ([C.c_int] if prefix == "rc" else []) + [C.POINTER(vp)])
    f("create").restype = C.c_int
    f("step").argtypes = [vp, C.c_int, C.POINTER(RcStepStats)]
    f("step").restype = C.c_int
    f("set_phase").argtypes = [vp, C.c_int]
    f("set_phase").restype = C.c_int
    f("get_sizes").argtypes = [vp, IP, IP, IP]
    f("get_sizes").restype = C.c_int
    f("download").argtypes = [vp, C.POINTER(RcCellHost), C.c_uint]
    f("download").restype = C.c_int
    f("site_count").argtypes = [vp]
    f("site_count").restype = C.c_longlong
    f("last_error").argtypes = [vp]
    f("last_error").restype = C.c_char_p
    f("destroy").argtypes = [vp]
    f("destroy").restype = None
    if prefix == "rc":
        lib.rc_upload.argtypes = [vp, C.POINTER(RcCellHost), C.c_uint]
        lib.rc_upload.restype = C.c_int
        lib.rc_set_stream.argtypes = [vp, vp]
        lib.rc_set_stream.restype = C.c_int
        lib.rc_abi_version.argtypes = []
        lib.rc_abi_version.restype = C.c_int
        lib.rc_step_async.argtypes = [vp, C.c_int]
        lib.rc_step_async.restype = C.c_int
        lib.rc_wait.argtypes = [vp, C.POINTER(RcStepStats)]
        lib.rc_wait.restype = C.c_int
        lib.rc_download_phi.argtypes = [vp, DP, C.c_longlong]
        lib.rc_download_phi.restype = C.c_int
        lib.rc_upload_phi.argtypes = [vp, DP, C.c_longlong]
        lib.rc_upload_phi.restype = C.c_int
        lib.rc_batch_create.argtypes = [C.POINTER(RcParams), C.c_int, C.POINTER(RcBox), C.POINTER(C.c_int),
                                        C.POINTER(RcCellHost), C.POINTER(C.c_ulonglong), C.c_int, C.POINTER(vp)]
        lib.rc_batch_create.restype = C.c_int
        lib.rc_create_generated.argtypes = [C.POINTER(RcParams), C.POINTER(RcBox), C.c_int, C.POINTER(RcCellHost),
                                            C.POINTER(RcGenerateSpec), C.c_int, C.POINTER(vp)]
        lib.rc_create_generated.restype = C.c_int
        lib.rc_layer_count.argtypes = [vp]
        lib.rc_layer_count.restype = C.c_int
        lib.rc_learned_harvest.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        lib.rc_learned_harvest.restype = C.c_int
        lib.rc_learned_harvested.argtypes = [vp]
        lib.rc_learned_harvested.restype = C.c_int
        lib.rc_learned_train.argtypes = [vp, C.POINTER(RcTrainOptions), C.POINTER(RcTrainReport)]
        lib.rc_learned_train.restype = C.c_int
        lib.rc_learned_get_params.argtypes = [vp, DP]
        lib.rc_learned_get_params.restype = C.c_int
        lib.rc_learned_set_params.argtypes = [vp, DP]
        lib.rc_learned_set_params.restype = C.c_int
        lib.rc_observe_field.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, DP, DP, DP, DP]
        lib.rc_observe_field.restype = C.c_int
        lib.rc_observe_stress.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, DP, DP, DP]
        lib.rc_observe_stress.restype = C.c_int
        lib.rc_observe_cells.argtypes = [vp, DP, DP]
        lib.rc_observe_cells.restype = C.c_int
        lib.rc_solver_profile.argtypes = [vp, C.c_int, DP, C.c_int]
        lib.rc_solver_profile.restype = C.c_int
        lib.rc_set_solver.argtypes = [vp, C.c_int]
        lib.rc_set_solver.restype = C.c_int
        lib.rc_unet_forward_tc.argtypes = [C.c_int, C.c_int, DP, DP, DP, C.c_int]
        lib.rc_unet_forward_tc.restype = C.c_int
        lib.rc_unet_loss_grad.argtypes = [C.c_int, C.c_int, DP, DP, DP, DP, DP, DP, C.c_int]
        lib.rc_unet_loss_grad.restype = C.c_int
        lib.rc_viscous_resolve_noalloc.argtypes = [vp, vp, vp, C.c_longlong, C.POINTER(C.c_int)]
        lib.rc_viscous_resolve_noalloc.restype = C.c_int
        lib.rc_viscous_resolve.argtypes = [vp, C.c_int, vp, vp, C.c_longlong, C.POINTER(RcStepStats)]
        lib.rc_viscous_resolve.restype = C.c_int
        lib.rc_set_cg_limits.argtypes = [vp, C.c_longlong, C.c_int]
        lib.rc_set_cg_limits.restype = C.c_int
        lib.rc_set_cg_tolerance.argtypes = [vp, C.c_double]
        lib.rc_set_cg_tolerance.restype = C.c_int
        lib.rc_test_barrier_timeout.argtypes = [vp, C.c_longlong, C.c_int]
        lib.rc_test_barrier_timeout.restype = C.c_int
        lib.rc_autotune.argtypes = [vp, C.c_int, C.POINTER(RcAutotuneReport)]
        lib.rc_autotune.restype = C.c_int
        lib.rc_set_cell_threads.argtypes = [vp, C.c_int]
        lib.rc_set_cell_threads.restype = C.c_int
        lib.rc_set_timing.argtypes = [vp, C.c_int]
        lib.rc_set_timing.restype = C.c_int
        lib.rc_timers.argtypes = [vp, DP, C.POINTER(C.c_longlong), C.c_int]
        lib.rc_timers.restype = C.c_int
        FP = C.POINTER(C.c_float)
        lib.rc_selftest_conversions.argtypes = [DP, FP, FP, FP, DP, C.c_longlong, C.c_int]
        lib.rc_selftest_conversions.restype = C.c_int
    else:
        lib.orc_rng_state.argtypes = [vp]
        lib.orc_rng_state.restype = C.c_ulonglong
    return lib


# Every symbol the header declares (checked by the CPU test suite).
EXPORTED = ["rc_abi_version", "rc_create", "rc_create_generated", "rc_batch_create", "rc_layer_count", "rc_viscous_resolve_noalloc", "rc_unet_loss_grad", "rc_unet_forward_tc",
            "rc_learned_harvest", "rc_learned_harvested", "rc_learned_train", "rc_learned_get_params",
            "rc_learned_set_params", "rc_set_solver", "rc_solver_profile", "rc_viscous_resolve",
            "rc_set_cg_limits", "rc_set_cg_tolerance", "rc_test_barrier_timeout",
            "rc_observe_field", "rc_observe_stress", "rc_observe_cells", "rc_autotune", "rc_set_cell_threads", "rc_step", "rc_step_async", "rc_wait", "rc_set_phase",
            "rc_get_sizes", "rc_download", "rc_upload", "rc_download_phi", "rc_upload_phi", "rc_set_stream",
            "rc_set_timing", "rc_timers", "rc_site_count", "rc_last_error", "rc_destroy",
            "rc_selftest_conversions"]

TIMER_NAMES = ["update", "gather", "forces", "solve", "repack", "rng", "epilogue"]
NUM_TIMERS = len(TIMER_NAMES)
