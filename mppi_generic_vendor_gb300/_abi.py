"""ctypes mirror of include/mppi_gb.h and the loader for libmppi_gb.so.

The library is the only compute path: if it is missing or fails to load, every call raises.  There is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

MPPI_MAX_STATE_DIM = 8
MPPI_MAX_CONTROL_DIM = 4
MPPI_MAX_OBSTACLES = 8

MPPI_OK = 0
MPPI_EINVAL, MPPI_ECUDA, MPPI_ENAN, MPPI_ETIMEOUT, MPPI_ENOMEM, MPPI_EUNSUPPORTED = 1, 2, 3, 4, 5, 6
STATUS_NAMES = {0: "MPPI_OK", 1: "MPPI_EINVAL", 2: "MPPI_ECUDA", 3: "MPPI_ENAN", 4: "MPPI_ETIMEOUT",
                5: "MPPI_ENOMEM", 6: "MPPI_EUNSUPPORTED"}

MODEL_CARTPOLE = 1
MODEL_DOUBLE_INTEGRATOR = 2
MODEL_BICYCLE_COSTMAP = 3
MODEL_BICYCLE_SLIP = 4
MODEL_BICYCLE_SLIP_MLP = 5
MODEL_PLUGIN = 100

SAMPLER_GAUSSIAN = 0
CONTROLLER_VANILLA, CONTROLLER_COLORED, CONTROLLER_TUBE, CONTROLLER_RMPPI = 0, 1, 2, 3
SAMPLER_COLORED_NOISE = 1

_F4 = C.c_float * MPPI_MAX_CONTROL_DIM
_FO = C.c_float * MPPI_MAX_OBSTACLES


class ControllerParams(C.Structure):
    _fields_ = [("dt", C.c_float), ("lambda_", C.c_float), ("alpha", C.c_float), ("num_timesteps", C.c_int),
                ("num_iters", C.c_int), ("seed", C.c_uint64), ("slide_control_scale", _F4), ("controller", C.c_int),
                ("tsallis_r", C.c_float), ("tsallis_gamma", C.c_float), ("leash_active", C.c_int),
                ("state_leash_dist", C.c_float * MPPI_MAX_STATE_DIM), ("nominal_threshold", C.c_float),
                ("value_function_threshold", C.c_float), ("num_candidate_nominal_states", C.c_int),
                ("num_eval_samples_per_candidate", C.c_int)]


class SamplingParams(C.Structure):
    _fields_ = [("kind", C.c_int), ("std_dev", _F4), ("control_cost_coeff", _F4),
                ("pure_noise_trajectories_percentage", C.c_float), ("std_dev_decay", C.c_float),
                ("exponents", _F4), ("offset_decay_rate", C.c_float), ("fmin", C.c_float),
                ("use_same_noise_for_all_distributions", C.c_int)]


class ControlConstraints(C.Structure):
    _fields_ = [("lower", _F4), ("upper", _F4), ("deadband", _F4), ("zero_control", _F4)]


class CartpoleParams(C.Structure):
    _fields_ = [("cart_mass", C.c_float), ("pole_mass", C.c_float), ("pole_length", C.c_float),
                ("gravity", C.c_float)]


class CartpoleCostParams(C.Structure):
    _fields_ = [("x_coeff", C.c_float), ("x_dot_coeff", C.c_float), ("cos_coeff", C.c_float),
                ("theta_dot_coeff", C.c_float), ("terminal_coeff", C.c_float)]


class DoubleIntegratorParams(C.Structure):
    _fields_ = [("reserved", C.c_float)]


class DIObstacleCostParams(C.Structure):
    _fields_ = [("goal", C.c_float * 4), ("coeff", C.c_float * 4), ("terminal_coeff", C.c_float),
                ("num_obstacles", C.c_int), ("obstacle_x", _FO), ("obstacle_y", _FO), ("obstacle_radius", _FO),
                ("obstacle_cost", C.c_float)]


class BicycleParams(C.Structure):
    _fields_ = [("wheelbase", C.c_float)]


class CostmapCostParams(C.Structure):
    _fields_ = [("map_coeff", C.c_float), ("speed_target", C.c_float), ("speed_coeff", C.c_float),
                ("steer_coeff", C.c_float), ("terminal_coeff", C.c_float)]


class BicycleSlipParams(C.Structure):
    _fields_ = [("mass", C.c_float), ("yaw_inertia", C.c_float), ("lf", C.c_float), ("lr", C.c_float),
                ("cornering_stiffness", C.c_float), ("max_drive_force", C.c_float), ("drag", C.c_float),
                ("max_steer", C.c_float), ("steer_time_constant", C.c_float), ("min_vx", C.c_float)]


MODEL_PARAM_TYPES = {
    MODEL_CARTPOLE: (CartpoleParams, CartpoleCostParams),
    MODEL_DOUBLE_INTEGRATOR: (DoubleIntegratorParams, DIObstacleCostParams),
    MODEL_BICYCLE_COSTMAP: (BicycleParams, CostmapCostParams),
    MODEL_BICYCLE_SLIP: (BicycleSlipParams, CostmapCostParams),
    MODEL_BICYCLE_SLIP_MLP: (BicycleSlipParams, CostmapCostParams),
}

_P = C.c_void_p
_FP = C.POINTER(C.c_float)
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)

# (name, restype, argtypes) for every exported function of include/mppi_gb.h
SIGNATURES = [
    ("mppi_abi_version", C.c_int, []),
    ("mppi_model_dims", C.c_int, [C.c_int, _IP, _IP, _IP]),
    ("mppi_model_param_sizes", C.c_int, [C.c_int, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    ("mppi_default_controller_params", None, [C.POINTER(ControllerParams)]),
    ("mppi_default_sampling_params", None, [C.POINTER(SamplingParams)]),
    ("mppi_default_constraints", None, [C.POINTER(ControlConstraints)]),
    ("mppi_last_error_string", C.c_char_p, []),
    ("mppi_create", C.c_int, [C.c_int, C.c_int, _IP, _IP, C.POINTER(ControllerParams), C.POINTER(SamplingParams),
                              C.POINTER(ControlConstraints), _P, C.c_size_t, _P, C.c_size_t, _FP, _P,
                              C.POINTER(_P)]),
    ("mppi_destroy", C.c_int, [_P]),
    ("mppi_get_instance_dims", C.c_int, [_P, C.c_int, _IP, _IP]),
    ("mppi_compute_control", C.c_int, [_P, _FP, C.c_int]),
    ("mppi_get_control_seq", C.c_int, [_P, _FP]),
    ("mppi_set_control_seq", C.c_int, [_P, _FP]),
    ("mppi_slide_control_sequence", C.c_int, [_P, C.c_int]),
    ("mppi_get_state_seq", C.c_int, [_P, _FP]),
    ("mppi_get_baseline_normalizer", C.c_int, [_P, _FP, _DP]),
    ("mppi_get_sample_costs", C.c_int, [_P, _FP]),
    ("mppi_get_sample_weights", C.c_int, [_P, _FP]),
    ("mppi_get_control_samples", C.c_int, [_P, _FP]),
    ("mppi_get_sampled_trajectories", C.c_int, [_P, C.c_int, C.POINTER(C.c_int), C.c_int, _FP, _FP, _FP, _IP]),
    ("mppi_get_model_dims", C.c_int, [_P, _IP, _IP, _IP, _IP]),
    ("mppi_get_nominal_state_used", C.c_int, [_P, _IP]),
    ("mppi_rmppi_update_importance_sampler", C.c_int, [_P, _FP, C.c_int]),
    ("mppi_rmppi_get_candidates", C.c_int, [_P, _IP, _IP, _FP, _IP, _FP, _FP]),
    ("mppi_set_feedback_params", C.c_int, [_P, _FP, _FP, _FP, C.c_int]),
    ("mppi_enable_feedback", C.c_int, [_P, C.c_int]),
    ("mppi_get_feedback_enabled", C.c_int, [_P, _IP]),
    ("mppi_compute_feedback", C.c_int, [_P, _FP]),
    ("mppi_get_feedback_gains", C.c_int, [_P, _FP]),
    ("mppi_get_feedback_control", C.c_int, [_P, _FP, _FP, C.c_int, _FP]),
    ("mppi_get_feedback_propagated_state_seq", C.c_int, [_P, _FP]),
    ("mppi_ddp_feedback_gains", C.c_int, [C.c_int, _P, C.c_size_t, C.c_int, C.c_float, _FP, _FP, _FP, _FP, _FP, _FP,
                                          C.c_int, _FP, _FP, _FP]),
    ("mppi_set_wait_diagnostics", C.c_int, [_P, C.c_uint32, C.c_int]),
    ("mppi_handle_adopt", C.c_int, [_P, C.c_int, C.POINTER(_P)]),
    ("mppi_select_top_samples", C.c_int, [_FP, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    ("mppi_get_free_energy", C.c_int, [_P, C.c_int, _FP]),
    ("mppi_set_dynamics_params", C.c_int, [_P, _P, C.c_size_t]),
    ("mppi_set_cost_params", C.c_int, [_P, _P, C.c_size_t]),
    ("mppi_set_sampling_params", C.c_int, [_P, C.POINTER(SamplingParams)]),
    ("mppi_set_controller_params", C.c_int, [_P, C.POINTER(ControllerParams)]),
    ("mppi_set_costmap", C.c_int, [_P, _FP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float]),
    ("mppi_set_mlp", C.c_int, [_P, _FP, C.c_size_t, C.c_int]),
    ("mppi_set_judge", C.c_int, [_P, C.c_float]),
    ("mppi_set_rollout_mode", C.c_int, [_P, C.c_int]),
    ("mppi_get_rollout_mode", C.c_int, [_P, _IP, _IP]),
    ("mppi_get_judge_stats", C.c_int, [_P, _FP]),
    ("mppi_use_analytic_dynamics", C.c_int, [_P, C.c_int]),
    ("mppi_inject_noise", C.c_int, [_P, _FP, C.c_size_t]),
    ("mppi_generate_samples", C.c_int, [_P, C.c_int, C.c_int]),
    ("mppi_set_graph_mode", C.c_int, [_P, C.c_int]),
    ("mppi_autotune", C.c_int, [_P, C.c_char_p]),
    ("mppi_get_launch_config", C.c_int, [_P, _IP, _IP, _IP]),
    ("mppi_set_launch_config", C.c_int, [_P, C.c_int, C.c_int, C.c_int]),
    ("mppi_kernels_per_compute", C.c_int, [_P, _IP]),
    ("mppi_enqueue_solve", C.c_int, [_P, C.c_int, C.c_int]),
    ("mppi_synchronize", C.c_int, [_P]),
    ("mppi_time_kernels", C.c_int, [_P, C.c_int, C.c_int, _FP]),
    ("mppi_get_stream", C.c_void_p, [_P]),
    ("mppi_kernel_weight_transform", C.c_int, [_P, _P, C.c_float, C.c_int, C.c_int, _P]),
    ("mppi_kernel_weighted_reduction", C.c_int, [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    ("mppi_kernel_weighted_reduction_noalloc", C.c_int, [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    ("mppi_kernel_rollout", C.c_int, [C.c_int, _P, C.c_size_t, _P, C.c_size_t, C.POINTER(SamplingParams), _P, _P,
                                      _P, _P, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _P]),
    ("mppi_kernel_gaussian_controls", C.c_int, [_P, _P, _FP, C.POINTER(ControlConstraints), C.c_int, C.c_int,
                                                C.c_int, C.c_int, C.c_float, C.c_float, _P]),
    ("mppi_kernel_philox_normal", C.c_int, [_P, C.c_size_t, C.c_uint64, C.c_uint64, _P]),
    ("mppi_kernel_philox_raw", C.c_int, [_P, C.c_size_t, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), _P]),
    ("mppi_kernel_sincos", C.c_int, [_P, _P, _P, C.c_size_t, _P]),
]

MLP_WEIGHTS = 5125
MLP_PARAMS = 5153


class SurrogateConfig(C.Structure):
    _fields_ = [("num_transitions", C.c_int), ("state_lower", C.c_float * 7), ("state_upper", C.c_float * 7),
                ("seed", C.c_uint64)]


SIGNATURES += [
    ("mppi_default_surrogate_config", None, [C.POINTER(SurrogateConfig)]),
    ("mppi_surrogate_create", C.c_int, [C.POINTER(BicycleSlipParams), C.POINTER(SurrogateConfig), _P,
                                        C.POINTER(_P)]),
    ("mppi_surrogate_destroy", C.c_int, [_P]),
    ("mppi_surrogate_generate", C.c_int, [_P]),
    ("mppi_surrogate_train", C.c_int, [_P, C.c_int, C.c_int, C.c_float, C.c_float, _FP]),
    ("mppi_surrogate_set_weight_format", C.c_int, [_P, C.c_int]),
    ("mppi_surrogate_gradient", C.c_int, [_P, _FP, _FP, C.c_int, _FP, _FP]),
    ("mppi_surrogate_validate", C.c_int, [_P, C.c_int, _FP]),
    ("mppi_surrogate_get_params", C.c_int, [_P, _FP]),
    ("mppi_surrogate_set_params", C.c_int, [_P, _FP]),
    ("mppi_kernel_mlp_forward", C.c_int, [_FP, C.c_int, _P, _P, C.c_int, _P]),
    ("mppi_mlp_quantize", C.c_int, [_FP, C.c_int, _FP, _FP]),
]

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "_build" / "libmppi_gb.so"
HEADER_PATH = PKG_DIR.parent / "include" / "mppi_gb.h"

_lib = None


class MPPIError(RuntimeError):
    """Raised when a C-ABI call returns a status other than MPPI_OK."""

    def __init__(self, status: int, func: str, message: str):
        self.status = status
        super().__init__(f"{func} -> {STATUS_NAMES.get(status, status)}: {message}")


def lib():
    """Load libmppi_gb.so (it must have been built; there is no fallback)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m mppi_generic_vendor_gb300.build` "
                               "(the engine has no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int, func: str = "mppi call"):
    if status != MPPI_OK:
        msg = lib().mppi_last_error_string()
        raise MPPIError(status, func, msg.decode() if msg else "")


def call(name: str, *args):
    """Call an exported function and raise MPPIError on a non-OK status."""
    st = getattr(lib(), name)(*args)
    check(st, name)
    return st


def default_controller_params(native: bool = True) -> ControllerParams:
    """ControllerParams defaults (controller.cuh:46-68).  native=False fills them without loading the engine library
    (for code that must not map it, such as the CPU baseline); a CPU test keeps both forms equal."""
    p = ControllerParams()
    if native:
        lib().mppi_default_controller_params(C.byref(p))
    else:
        p.dt, p.lambda_, p.alpha, p.num_timesteps, p.num_iters, p.seed = 0.02, 1.0, 0.0, 100, 1, 0
        p.controller, p.tsallis_r, p.tsallis_gamma, p.leash_active = CONTROLLER_VANILLA, 2.0, 0.0, 0
        p.nominal_threshold = 20.0
        p.value_function_threshold, p.num_candidate_nominal_states, p.num_eval_samples_per_candidate = 1000.0, 9, 64
    return p


def default_sampling_params(native: bool = True) -> SamplingParams:
    """GaussianParamsImpl / ColoredNoiseParamsImpl defaults (gaussian.cuh:21-61, colored_noise.cuh:44-73)."""
    p = SamplingParams()
    if native:
        lib().mppi_default_sampling_params(C.byref(p))
    else:
        p.kind = 0
        for i in range(MPPI_MAX_CONTROL_DIM):
            p.std_dev[i] = 1.0
        p.pure_noise_trajectories_percentage = 0.01
        p.std_dev_decay = 1.0
        p.offset_decay_rate = 0.97
        p.fmin = 0.0
        p.use_same_noise_for_all_distributions = 1
    return p


def default_constraints(native: bool = True) -> ControlConstraints:
    """Unbounded control ranges (Dynamics::setDefaultControlRanges, dynamics.cu:19-26)."""
    c = ControlConstraints()
    if native:
        lib().mppi_default_constraints(C.byref(c))
    else:
        flt_max = 3.4028234663852886e38  # FLT_MAX
        for i in range(MPPI_MAX_CONTROL_DIM):
            c.lower[i], c.upper[i], c.deadband[i], c.zero_control[i] = -flt_max, flt_max, 0.0, 0.0
    return c
