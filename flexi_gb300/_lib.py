"""ctypes binding of libflexigpu.so (C ABI in include/flexi_gpu.h)."""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libflexigpu.so")
_lib = None


class FgConfig(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("NodeType", ctypes.c_int), ("Riemann", ctypes.c_int), ("RiemannBC", ctypes.c_int),
                ("Lifting", ctypes.c_int), ("doWeakLifting", ctypes.c_int), ("doConservativeLifting", ctypes.c_int),
                ("SplitDG", ctypes.c_int), ("etaBR2", ctypes.c_double), ("etaBR2_wall", ctypes.c_double), ("kappa", ctypes.c_double),
                ("R", ctypes.c_double), ("Pr", ctypes.c_double), ("mu0", ctypes.c_double), ("CFLScale", ctypes.c_double),
                ("DFLScale", ctypes.c_double), ("doTCSource", ctypes.c_int), ("dpdx", ctypes.c_double), ("TimeDiscMethod", ctypes.c_int),
                ("OverintegrationType", ctypes.c_int), ("NUnder", ctypes.c_int), ("IniExactFunc", ctypes.c_int),
                ("AdvVel", ctypes.c_double * 3), ("IniFrequency", ctypes.c_double), ("IniAmplitude", ctypes.c_double),
                ("TEnd", ctypes.c_double), ("Analyze_dt", ctypes.c_double), ("dtmin", ctypes.c_double), ("dtkill", ctypes.c_double),
                ("nCalcTimeStepMax", ctypes.c_int), ("maxIter", ctypes.c_int), ("RiemannPhiFactor", ctypes.c_double)]


class FgTimeDiscState(ctypes.Structure):
    """fg_timedisc_state: per-instance state of the time loop."""
    _fields_ = [("t", ctypes.c_double), ("dt", ctypes.c_double), ("dtMin", ctypes.c_double), ("iter", ctypes.c_longlong),
                ("atAnalyze", ctypes.c_int), ("finished", ctypes.c_int), ("nDtLimited", ctypes.c_int)]


EXPORTS = ["fg_config_default", "fg_config_from_ini", "fg_create", "fg_destroy", "fg_last_error", "fg_build_mesh", "fg_build_mesh_mortar", "fg_set_mesh", "fg_set_mesh_mortar", "fg_set_face_metrics", "fg_overintegrate_state",
           "fg_get_config", "fg_lserk_table", "fg_set_time", "fg_hopr_sizes", "fg_hopr_read", "fg_write_state", "fg_read_state", "fg_io_last_error",
           "fg_set_instance_mu0", "fg_get_elem_xgp", "fg_get_sizes", "fg_get_mesh_array", "fg_get_side_to_elem", "fg_set_state",
           "fg_get_state", "fg_state_device_ptr", "fg_time_derivative", "fg_calc_timestep", "fg_get_dt_elem", "fg_timestep_lserkw2", "fg_run", "fg_run_to_host",
           "fg_get_gradients", "fg_get_stream", "fg_launch_count", "fg_get_timedisc_state", "fg_debug_array", "fg_profile_enable", "fg_profile_read", "fg_probe_fp64", "fg_probe_fp64_pipe", "fg_probe_fp64_tensor", "fg_probe_fp64_lanes",
           "fg_time_derivative_noalloc", "fg_set_elem_mu_scale", "fg_vjp_time_derivative", "fg_adjoint_forward", "fg_adjoint_reverse",
           "fg_set_body_force_field", "fg_wall_shear", "fg_jvp_time_derivative",
           "fg_adjoint_recomputed_steps", "fg_autotune", "fg_autotune_choice",
           "fg_set_launch_shapes"]


class FgDeviceMesh(ctypes.Structure):
    """fg_device_mesh: caller-owned device arrays for fg_time_derivative_noalloc (pointers as integers)."""
    _fields_ = [("nElems", ctypes.c_int), ("nSides", ctypes.c_int), ("nBCSides", ctypes.c_int),
                ("elemSide", ctypes.c_void_p), ("sideElem", ctypes.c_void_p), ("metr", ctypes.c_void_p), ("sJ", ctypes.c_void_p),
                ("geo", ctypes.c_void_p), ("bcType", ctypes.c_void_p), ("bcTwall", ctypes.c_void_p)]


def load(path=None):
    """Loads the library; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libflexigpu.so not found at {path}; run __graft_entry__.build() (no CPU fallback exists)")
    L = ctypes.CDLL(path)
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    PI = ctypes.POINTER(ctypes.c_int)
    L.fg_config_default.argtypes = [ctypes.POINTER(FgConfig)]
    L.fg_config_from_ini.argtypes = [ctypes.c_char_p, ctypes.POINTER(FgConfig)]
    L.fg_create.argtypes = [ctypes.POINTER(FgConfig), ctypes.POINTER(P)]
    L.fg_destroy.argtypes = [P]
    L.fg_last_error.argtypes = [P]
    L.fg_last_error.restype = ctypes.c_char_p
    L.fg_build_mesh.argtypes = [P, I, I, P, P, I, P, I, P, P]
    L.fg_build_mesh_mortar.argtypes = [P, I, I, P, P, I, P, I, P, P, I, P]
    L.fg_set_mesh.argtypes = [P, I, I, I, P, P, P, I, P, I, P, P, P, P, P, P, P, P, P]
    L.fg_set_mesh_mortar.argtypes = [P, I, I, I, P, P, P, I, P, I, P, P, P, P, P, P, P, P, P, I, P, P]
    L.fg_set_face_metrics.argtypes = [P, P, P]
    L.fg_overintegrate_state.argtypes = [P]
    L.fg_get_config.argtypes = [P, P]
    L.fg_lserk_table.argtypes = [I, P, P, P, P, P, P]
    L.fg_set_time.argtypes = [P, P]
    L.fg_hopr_sizes.argtypes = [ctypes.c_char_p, P]
    L.fg_hopr_read.argtypes = [ctypes.c_char_p, P, P, P, P, P]
    L.fg_write_state.argtypes = [P, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_double]
    L.fg_read_state.argtypes = [P, ctypes.c_char_p, P]
    L.fg_io_last_error.restype = ctypes.c_char_p
    L.fg_io_last_error.argtypes = []
    L.fg_set_instance_mu0.argtypes = [P, I, P]
    L.fg_get_elem_xgp.argtypes = [P, P]
    L.fg_get_sizes.argtypes = [P, P]
    L.fg_get_mesh_array.argtypes = [P, I, P]
    L.fg_get_side_to_elem.argtypes = [P, P]
    L.fg_set_state.argtypes = [P, P]
    L.fg_get_state.argtypes = [P, P]
    L.fg_state_device_ptr.argtypes = [P, ctypes.POINTER(P)]
    L.fg_time_derivative.argtypes = [P, D, P]
    L.fg_calc_timestep.argtypes = [P, P, PI]
    L.fg_get_dt_elem.argtypes = [P, P, P]
    L.fg_timestep_lserkw2.argtypes = [P, ctypes.POINTER(D), D]
    L.fg_run.argtypes = [P, I, P]
    L.fg_run_to_host.argtypes = [P, I, P, P]
    L.fg_get_timedisc_state.argtypes = [P, I, P]
    L.fg_probe_fp64_pipe.argtypes = [P]
    L.fg_probe_fp64_tensor.argtypes = [P]
    L.fg_probe_fp64_lanes.argtypes = [P]
    L.fg_get_gradients.argtypes = [P, P, P, P]
    L.fg_get_stream.argtypes = [P, ctypes.POINTER(P)]
    L.fg_launch_count.argtypes = [P]
    L.fg_launch_count.restype = ctypes.c_longlong
    L.fg_debug_array.argtypes = [P, ctypes.c_char_p, P, ctypes.POINTER(ctypes.c_longlong)]
    L.fg_profile_enable.argtypes = [P, I]
    L.fg_profile_read.argtypes = [P, P, P]
    L.fg_probe_fp64.argtypes = [ctypes.POINTER(D)]
    L.fg_set_elem_mu_scale.argtypes = [P, P]
    L.fg_vjp_time_derivative.argtypes = [P, D, P, P, P]
    L.fg_jvp_time_derivative.argtypes = [P, D, P, P, I, I, D]
    L.fg_adjoint_forward.argtypes = [P, I, D, I]
    L.fg_adjoint_reverse.argtypes = [P, P, P, P, P]
    L.fg_adjoint_recomputed_steps.argtypes = [P]
    L.fg_autotune.argtypes = [P, I, P]
    L.fg_autotune_choice.argtypes = [P, P]
    L.fg_set_launch_shapes.argtypes = [P, I, I, I, I]
    L.fg_adjoint_recomputed_steps.restype = ctypes.c_longlong
    L.fg_set_body_force_field.argtypes = [P, P]
    L.fg_wall_shear.argtypes = [P, P, P]
    L.fg_time_derivative_noalloc.argtypes = [ctypes.POINTER(FgConfig), ctypes.POINTER(FgDeviceMesh), P, P, P]
    _lib = L
    return L
