"""Host-side mirror of MPPI-Generic's plugin and controller interface over the C ABI.

Names, argument meanings and shapes follow the reference so that code written against it reads the same:

* plugins — ``CartpoleDynamics``, ``DoubleIntegratorDynamics``, ``BicycleDynamics``, ``BicycleSlipDynamics``
  (Dynamics, include/mppi/dynamics/dynamics.cuh:68), the matching costs (Cost, cost_functions/cost.cuh:34) and
  ``GaussianDistribution`` / ``ColoredNoiseDistribution`` (sampling_distributions/gaussian/gaussian.cuh:98,
  colored_noise/colored_noise.cuh:79);
* ``VanillaMPPIController`` (controllers/MPPI/mppi_controller.cuh:14) with ``computeControl``, ``getControlSeq``,
  ``slideControlSequence``, ``getBaselineCost``, ``getNormalizerCost``, ``getSampledCostSeq``,
  ``getTargetStateSeq``, ``setParams`` / ``getParams``;
* ``BatchedMPPIController``: many independent controllers of one plugin pair, solved together on the GPU.

Control and state sequences are returned as (C, T) / (S, T) arrays, the shape of the reference's column-major Eigen
trajectories.  All compute runs in libmppi_gb.so; nothing here computes MPPI on the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A


def _fptr(a: np.ndarray):
    """float* of a float32 array.  A ctypes array over the array's own buffer costs under a microsecond, against
    several for ndarray.ctypes.data_as, which matters on the per-iteration calls; read-only or strided arrays take
    the general route."""
    if a.dtype == np.float32 and a.flags.c_contiguous and a.flags.writeable and a.size > 0:
        return (C.c_float * a.size).from_buffer(a)
    return a.ctypes.data_as(C.POINTER(C.c_float))


def select_top_samples(weights, n):
    """Controller::copyTopControlFromDevice's selection (controller.cu:126-181): indices of the n highest weights by the
    reference's replacement scan, in its list order."""
    w = np.ascontiguousarray(weights, dtype=np.float32)
    out = np.empty(int(n), dtype=np.int32)
    A.call("mppi_select_top_samples", _fptr(w), int(w.size), int(n), out.ctypes.data_as(C.POINTER(C.c_int)))
    return out


# ------------------------------------------------------------------------------------------------------ plugins
class _Plugin:
    model_id: int = 0

    def __init__(self, params):
        self.params_ = params

    def getParams(self):
        return self.params_

    def setParams(self, params):
        self.params_ = params


class CartpoleDynamics(_Plugin):
    """CartpoleDynamics(cart_mass, pole_mass, pole_length) (dynamics/cartpole/cartpole_dynamics.cu:4-8)."""

    model_id = A.MODEL_CARTPOLE
    STATE_DIM, CONTROL_DIM, OUTPUT_DIM = 4, 1, 4

    def __init__(self, cart_mass=1.0, pole_mass=1.0, pole_length=1.0, gravity=9.81):
        super().__init__(A.CartpoleParams(cart_mass, pole_mass, pole_length, gravity))
        self.control_rngs = [(-np.finfo(np.float32).max, np.finfo(np.float32).max)]

    def setControlRanges(self, ranges):
        self.control_rngs = [tuple(r) for r in ranges]


class CartpoleSwingupCost(_Plugin):
    """x_coeff x^2 + x_dot_coeff xdot^2 + cos_coeff (1 + cos theta)^2 + theta_dot_coeff thetadot^2."""

    def __init__(self, x_coeff=10.0, x_dot_coeff=1.0, cos_coeff=100.0, theta_dot_coeff=1.0, terminal_coeff=0.0):
        super().__init__(A.CartpoleCostParams(x_coeff, x_dot_coeff, cos_coeff, theta_dot_coeff, terminal_coeff))


class DoubleIntegratorDynamics(_Plugin):
    """DoubleIntegratorDynamics (dynamics/double_integrator/di_dynamics.cu:46-53)."""

    model_id = A.MODEL_DOUBLE_INTEGRATOR
    STATE_DIM, CONTROL_DIM, OUTPUT_DIM = 4, 2, 4

    def __init__(self):
        super().__init__(A.DoubleIntegratorParams(0.0))
        self.control_rngs = [(-np.finfo(np.float32).max, np.finfo(np.float32).max)] * 2

    def setControlRanges(self, ranges):
        self.control_rngs = [tuple(r) for r in ranges]


class DoubleIntegratorObstacleCost(_Plugin):
    """Weighted squared error to a goal state plus obstacle_cost inside any of up to 8 circles."""

    def __init__(self, goal=(0, 0, 0, 0), coeff=(1, 1, 0.1, 0.1), terminal_coeff=0.0, obstacles=(),
                 obstacle_cost=1000.0):
        p = A.DIObstacleCostParams()
        p.goal[:] = [float(v) for v in goal]
        p.coeff[:] = [float(v) for v in coeff]
        p.terminal_coeff = terminal_coeff
        obstacles = list(obstacles)
        if len(obstacles) > A.MPPI_MAX_OBSTACLES:
            raise ValueError(f"at most {A.MPPI_MAX_OBSTACLES} obstacles")
        p.num_obstacles = len(obstacles)
        for j, (x, y, r) in enumerate(obstacles):
            p.obstacle_x[j], p.obstacle_y[j], p.obstacle_radius[j] = x, y, r
        p.obstacle_cost = obstacle_cost
        super().__init__(p)


class BicycleDynamics(_Plugin):
    """Kinematic bicycle: state (x, y, yaw, v), control (accel, steer)."""

    model_id = A.MODEL_BICYCLE_COSTMAP
    STATE_DIM, CONTROL_DIM, OUTPUT_DIM = 4, 2, 4

    def __init__(self, wheelbase=2.5):
        super().__init__(A.BicycleParams(wheelbase))
        self.control_rngs = [(-3.0, 3.0), (-1.0, 1.0)]

    def setControlRanges(self, ranges):
        self.control_rngs = [tuple(r) for r in ranges]


class BicycleSlipDynamics(_Plugin):
    """Dynamic bicycle with linear tyres: state (x, y, yaw, vx, vy, yaw_rate, steer), control (throttle, steer_cmd)."""

    model_id = A.MODEL_BICYCLE_SLIP
    STATE_DIM, CONTROL_DIM, OUTPUT_DIM = 7, 2, 7

    def __init__(self, mass=1500.0, yaw_inertia=2500.0, lf=1.2, lr=1.3, cornering_stiffness=8e4,
                 max_drive_force=4000.0, drag=50.0, max_steer=0.5, steer_time_constant=0.1, min_vx=1.0):
        super().__init__(A.BicycleSlipParams(mass, yaw_inertia, lf, lr, cornering_stiffness, max_drive_force, drag,
                                             max_steer, steer_time_constant, min_vx))
        self.control_rngs = [(-1.0, 1.0), (-1.0, 1.0)]

    def setControlRanges(self, ranges):
        self.control_rngs = [tuple(r) for r in ranges]


class BicycleSlipMLPDynamics(BicycleSlipDynamics):
    """Dynamic bicycle whose five non-kinematic derivatives come from the learned 9-64-64-5 surrogate
    (NeuralNetModel, include/mppi/dynamics/autorally/ar_nn_model.cuh:133-145).  The network is evaluated on the
    tensor cores with BF16 (``precision="bf16"``) or FP8 E4M3 (``"fp8"``) weights and FP32 accumulation, or in plain
    FP32 on the CUDA cores (``"fp32"``, one thread per sample as the reference's FNNHelper).  The
    ``BicycleSlipDynamics`` parameters are kept for the analytic judge and the host twin."""

    model_id = A.MODEL_BICYCLE_SLIP_MLP
    PRECISIONS = {"bf16": 0, "fp8": 1, "fp32": 2}

    def __init__(self, params=None, precision="bf16", **slip_kwargs):
        super().__init__(**slip_kwargs)
        if precision not in self.PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(self.PRECISIONS)}")
        self.precision = precision
        self.mlp_params = None
        if params is not None:
            self.updateModel(params)

    def updateModel(self, params):
        """Network + normalisation parameters, MPPI_MLP_PARAMS floats (``Surrogate.params()``)."""
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(-1))
        if p.size != A.MLP_PARAMS:
            raise ValueError(f"surrogate parameter vector must hold {A.MLP_PARAMS} floats")
        self.mlp_params = p

    def loadParams(self, path, prefix=""):
        """Network from an npz file: a ``Surrogate.save`` checkpoint, or the reference's FNNHelper arrays
        ``dynamics_W{i}`` / ``dynamics_b{i}`` (FNNHelper::loadParams, fnn_helper.cu:64-127), which carry no
        normalisation (identity scaling)."""
        from . import nn_io

        self.updateModel(nn_io.load(path, prefix))


class CostmapCost(_Plugin):
    """map_coeff * bilinear(costmap, x, y) + speed_coeff (v - speed_target)^2 + steer_coeff steer^2."""

    def __init__(self, map_coeff=1.0, speed_target=8.0, speed_coeff=1.0, steer_coeff=0.0, terminal_coeff=0.0,
                 costmap=None, resolution=0.1, origin=(0.0, 0.0)):
        super().__init__(A.CostmapCostParams(map_coeff, speed_target, speed_coeff, steer_coeff, terminal_coeff))
        self.costmap = None if costmap is None else np.ascontiguousarray(costmap, dtype=np.float32)
        self.resolution = float(resolution)
        self.origin = (float(origin[0]), float(origin[1]))


@dataclass
class GaussianDistribution:
    """GaussianDistributionImpl parameters (sampling_distributions/gaussian/gaussian.cuh:21-61)."""

    std_dev: tuple = (1.0,)
    control_cost_coeff: tuple = (0.0,)
    pure_noise_trajectories_percentage: float = 0.01
    std_dev_decay: float = 1.0
    # SamplingParams::use_same_noise_for_all_distributions (sampling_distribution.cuh:20): Tube-MPPI's two
    # distributions draw the same standard normals
    use_same_noise_for_all_distributions: bool = True
    kind: int = field(default=A.SAMPLER_GAUSSIAN, init=False)

    def to_c(self) -> A.SamplingParams:
        p = A.default_sampling_params()
        p.kind = self.kind
        for i, v in enumerate(self.std_dev):
            p.std_dev[i] = v
        for i, v in enumerate(self.control_cost_coeff):
            p.control_cost_coeff[i] = v
        p.pure_noise_trajectories_percentage = self.pure_noise_trajectories_percentage
        p.std_dev_decay = self.std_dev_decay
        p.use_same_noise_for_all_distributions = int(bool(self.use_same_noise_for_all_distributions))
        return p


@dataclass
class ColoredNoiseDistribution(GaussianDistribution):
    """ColoredNoiseDistributionImpl parameters (sampling_distributions/colored_noise/colored_noise.cuh:44-73)."""

    exponents: tuple = (1.0,)
    offset_decay_rate: float = 0.97
    fmin: float = 0.0

    def __post_init__(self):
        self.kind = A.SAMPLER_COLORED_NOISE

    def to_c(self) -> A.SamplingParams:
        p = super().to_c()
        for i, v in enumerate(self.exponents):
            p.exponents[i] = v
        p.offset_decay_rate = self.offset_decay_rate
        p.fmin = self.fmin
        return p


# ------------------------------------------------------------------------------------------------ controllers
# ------------------------------------------------------------------------------------------- feedback controller
@dataclass
class DDPParams:
    """DDPParams (feedback_controllers/DDP/ddp.cuh:16-25): tracking weights Q, Q_f (S x S) and R (C x C) and the
    number of DDP iterations; None means the identity."""
    Q: np.ndarray | None = None
    Q_f: np.ndarray | None = None
    R: np.ndarray | None = None
    num_iterations: int = 1


@dataclass
class DDPFeedbackState:
    """DDPFeedbackState (ddp.cuh:28-37): the gain trajectory, per step a C x S matrix stored column-major."""
    fb_gain_traj_: np.ndarray
    state_dim: int
    control_dim: int

    def gain(self, t: int) -> np.ndarray:
        """K_t as a (C, S) array."""
        n = self.state_dim * self.control_dim
        return self.fb_gain_traj_[t * n:(t + 1) * n].reshape(self.state_dim, self.control_dim).T


class DDPFeedback:
    """DDPFeedback(model, dt, num_timesteps) (feedback_controllers/DDP/ddp.cuh:104-160): the ancillary controller a
    VanillaMPPIController / TubeMPPIController is built with.  It holds the DDPParams; the controller's handle runs the
    solver (mppi_compute_feedback) on the host after a solve."""

    def __init__(self, model, dt, num_timesteps=None):
        self.model_ = model
        self.dt_ = float(dt)
        self.num_timesteps_ = num_timesteps
        S, Cd = model.STATE_DIM, model.CONTROL_DIM
        self.params_ = DDPParams(np.eye(S, dtype=np.float32), np.eye(S, dtype=np.float32),
                                 np.eye(Cd, dtype=np.float32), 1)
        self._controllers = []

    def getParams(self) -> DDPParams:
        return DDPParams(*(None if m is None else np.array(m, np.float32) for m in
                           (self.params_.Q, self.params_.Q_f, self.params_.R)), self.params_.num_iterations)

    def setParams(self, params: DDPParams):
        """FeedbackController::setParams (ddp.cu:81-87); handed on to every controller built with this object."""
        self.params_ = params
        for c in self._controllers:
            c.setFeedbackParams(params)


def _col_major(m, n):
    """A float32 n x n matrix in column-major order (the reference's Eigen storage), or None for the identity."""
    if m is None:
        return None
    a = np.asarray(m, dtype=np.float32).reshape(n, n)
    return np.ascontiguousarray(a.T.reshape(-1))


class BatchedMPPIController:
    """Many independent VanillaMPPIControllers of one plugin pair, solved by one set of GPU launches.

    ``dynamics`` / ``costs`` are one plugin object each or a list with one per instance; ``num_rollouts`` and
    ``num_timesteps`` are per-instance sequences.  ``stream`` is a cudaStream_t as an int (0 = own stream).
    """

    def __init__(self, dynamics, costs, sampler, num_rollouts, num_timesteps, dt=0.02, max_iter=1, lambda_=1.0,
                 alpha=0.0, seed=0, init_control_traj=None, stream=0, slide_control_scale=None):
        self.num_instances = len(num_rollouts)
        dyn_list = dynamics if isinstance(dynamics, (list, tuple)) else [dynamics] * self.num_instances
        cost_list = costs if isinstance(costs, (list, tuple)) else [costs] * self.num_instances
        if len(dyn_list) != self.num_instances or len(cost_list) != self.num_instances:
            raise ValueError("one dynamics and one cost object per instance")
        self.model_ = dyn_list[0]
        self.cost_ = cost_list[0]
        self.sampler_ = sampler
        self.model_id = self.model_.model_id
        self.S, self.Cdim = self.model_.STATE_DIM, self.model_.CONTROL_DIM
        self.output_dim = getattr(self.model_, "OUTPUT_DIM", self.S)
        self.K = np.asarray(num_rollouts, dtype=np.int32)
        self.T = np.asarray(num_timesteps, dtype=np.int32)
        dyn_t, cost_t = type(dyn_list[0].getParams()), type(cost_list[0].getParams())
        self._dyn_arr = (dyn_t * self.num_instances)(*[d.getParams() for d in dyn_list])
        self._cost_arr = (cost_t * self.num_instances)(*[c.getParams() for c in cost_list])
        cp = A.default_controller_params()
        cp.dt, cp.lambda_, cp.alpha, cp.num_iters, cp.seed = dt, lambda_, alpha, max_iter, seed
        cp.num_timesteps = int(self.T.max())
        if slide_control_scale is not None:
            for i, v in enumerate(slide_control_scale):
                cp.slide_control_scale[i] = v
        self.params_ = cp
        cc = A.default_constraints()
        for i, (lo, hi) in enumerate(self.model_.control_rngs):
            cc.lower[i], cc.upper[i] = lo, hi
        self.constraints_ = cc
        self._t_off = np.concatenate([[0], np.cumsum(self.T * self.Cdim)]).astype(np.int64)
        self._s_off = np.concatenate([[0], np.cumsum(self.T * self.S)]).astype(np.int64)
        self._k_off = np.concatenate([[0], np.cumsum(self.K)]).astype(np.int64)
        init = None
        if init_control_traj is not None:
            init = np.ascontiguousarray(np.asarray(init_control_traj, dtype=np.float32).reshape(-1))
            if init.size != self._t_off[-1]:
                raise ValueError(f"init_control_traj must hold {self._t_off[-1]} floats")
        sp = sampler.to_c()
        self._h = self._create_handle(cp, sp, cc, None if init is None else _fptr(init), stream)
        cm = getattr(self.cost_, "costmap", None)
        if cm is not None:
            self.setCostmap(cm, self.cost_.resolution, self.cost_.origin)
        mlp = getattr(self.model_, "mlp_params", None)
        if mlp is not None:
            self.setMLP(mlp, self.model_.precision)

    def _create_handle(self, cp, sp, cc, init, stream):
        """mppi_create for a built-in model (VanillaMPPIController's constructor, mppi_controller.cu:16-29)."""
        h = C.c_void_p()
        dyn_t, cost_t = type(self._dyn_arr[0]), type(self._cost_arr[0])
        A.call("mppi_create", self.model_id, self.num_instances, self.K.ctypes.data_as(C.POINTER(C.c_int)),
               self.T.ctypes.data_as(C.POINTER(C.c_int)), C.byref(cp), C.byref(sp), C.byref(cc),
               C.cast(self._dyn_arr, C.c_void_p), C.sizeof(dyn_t), C.cast(self._cost_arr, C.c_void_p),
               C.sizeof(cost_t), init, C.c_void_p(stream or None), C.byref(h))
        return h

    # ---- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            A.lib().mppi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- the hot path
    def computeControl(self, state, optimization_stride=1):
        """VanillaMPPIController::computeControl (controllers/MPPI/mppi_controller.cu:152-237) for all instances."""
        x0 = np.ascontiguousarray(np.asarray(state, dtype=np.float32).reshape(-1))
        if x0.size != self.num_instances * self.S:
            raise ValueError(f"state must hold {self.num_instances * self.S} floats")
        A.call("mppi_compute_control", self._h, _fptr(x0), int(optimization_stride))

    def computeControlFlat(self, x0: np.ndarray, optimization_stride=1):
        """computeControl without reshaping or copying (x0 must be contiguous float32)."""
        A.call("mppi_compute_control", self._h, _fptr(x0), int(optimization_stride))

    # ---- accessors (flat, all instances)
    def control_flat(self) -> np.ndarray:
        out = np.empty(int(self._t_off[-1]), dtype=np.float32)
        A.call("mppi_get_control_seq", self._h, _fptr(out))
        return out

    def getControlSeqs(self):
        flat = self.control_flat()
        return [flat[self._t_off[i]:self._t_off[i + 1]].reshape(int(self.T[i]), self.Cdim).T.copy()
                for i in range(self.num_instances)]

    def setControlSeqs(self, seqs):
        flat = np.concatenate([np.asarray(s, dtype=np.float32).T.reshape(-1) for s in seqs])
        flat = np.ascontiguousarray(flat)
        A.call("mppi_set_control_seq", self._h, _fptr(flat))

    def updateImportanceSamplingControl(self, state, stride=1):
        """Controller::updateImportanceSamplingControl (controller.cuh:322-329): nothing here; the robust
        controller's replaces it.  The plant calls it before every slide (base_plant.hpp:536-540)."""

    def slideControlSequence(self, steps):
        """Controller::slideControlSequence (controllers/controller.cuh:370-376)."""
        A.call("mppi_slide_control_sequence", self._h, int(steps))

    def getTargetStateSeqs(self):
        out = np.empty(int(self._s_off[-1]), dtype=np.float32)
        A.call("mppi_get_state_seq", self._h, _fptr(out))
        return [out[self._s_off[i]:self._s_off[i + 1]].reshape(int(self.T[i]), self.S).T.copy()
                for i in range(self.num_instances)]

    def baseline_normalizer(self):
        out = np.empty(2 * self.num_instances, dtype=np.float32)
        n64 = np.empty(self.num_instances, dtype=np.float64)
        A.call("mppi_get_baseline_normalizer", self._h, _fptr(out), n64.ctypes.data_as(C.POINTER(C.c_double)))
        return out.reshape(-1, 2), n64

    def getBaselineCost(self, ind=0):
        return float(self.baseline_normalizer()[0][ind, 0])

    def getNormalizerCost(self, ind=0):
        return float(self.baseline_normalizer()[0][ind, 1])

    def sample_costs(self) -> np.ndarray:
        out = np.empty(int(self._k_off[-1]), dtype=np.float32)
        A.call("mppi_get_sample_costs", self._h, _fptr(out))
        return out

    def sample_weights(self) -> np.ndarray:
        out = np.empty(int(self._k_off[-1]), dtype=np.float32)
        A.call("mppi_get_sample_weights", self._h, _fptr(out))
        return out

    def control_samples(self) -> np.ndarray:
        n = int(np.sum(self.K.astype(np.int64) * self.T * self.Cdim))
        out = np.empty(n, dtype=np.float32)
        A.call("mppi_get_control_samples", self._h, _fptr(out))
        return out

    # ---- sampled trajectories for visualisation (Controller::setPercentageSampledControlTrajectoriesHelper,
    #      setTopNSampledControlTrajectoriesHelper, controller.cuh:754-767; calculateSampledStateTrajectories,
    #      getSampledOutputTrajectories, getSampledCostTrajectories, getTopTransformedCosts, controller.cuh:234-314)
    def setPercentageSampledControlTrajectories(self, perc):
        self._vis_perc = float(perc)

    def setTopNSampledControlTrajectories(self, n):
        self._vis_top = int(n)

    def calculateSampledStateTrajectories(self, instance=0, seed=0):
        """Re-roll on the GPU a random share of the last solve's samples (drawn without replacement from the first
        98%, copySampledControlFromDevice, controller.cu:57-105) followed by the top-N by weight
        (copyTopControlFromDevice's selection, controller.cu:126-181)."""
        i = int(instance)
        K, T = int(self.K[i]), int(self.T[i])
        perc, top_n = getattr(self, "_vis_perc", 0.0), getattr(self, "_vis_top", 0)
        n_rand = int(perc * K)
        if perc > 0.98:
            rand = np.arange(n_rand, dtype=np.int32)
        else:
            rand = np.random.default_rng(seed).choice(int(K * 0.98), n_rand, replace=False).astype(np.int32)
        w = self.sample_weights()[int(self._k_off[i]):int(self._k_off[i + 1])].copy()
        top = select_top_samples(w, top_n) if top_n > 0 else np.empty(0, np.int32)
        idx = np.ascontiguousarray(np.concatenate([rand, top]).astype(np.int32))
        n = idx.size
        O = self.output_dim
        states = np.empty(max(n, 1) * T * O, np.float32)
        step_costs = np.empty(max(n, 1) * T, np.float32)
        terminal = np.empty(max(n, 1), np.float32)
        crash = np.empty(max(n, 1) * T, np.int32)
        if n:
            A.call("mppi_get_sampled_trajectories", self._h, i, idx.ctypes.data_as(C.POINTER(C.c_int)), n,
                   _fptr(states), _fptr(step_costs), _fptr(terminal), crash.ctypes.data_as(C.POINTER(C.c_int)))
        self.sampled_indices_ = idx
        self.sampled_trajectories_ = [states[j * T * O:(j + 1) * T * O].reshape(T, O).T.copy() for j in range(n)]
        self.sampled_costs_ = [step_costs[j * T:(j + 1) * T].copy() for j in range(n)]
        self.sampled_crash_status_ = [crash[j * T:(j + 1) * T].copy() for j in range(n)]
        self.sampled_terminal_costs_ = terminal[:n].copy()
        self.top_n_costs_ = w[top] / self.getNormalizerCost(i) if top_n > 0 else np.empty(0, np.float32)

    def getSampledOutputTrajectories(self):
        """(S, T) state trajectory of each re-rolled sample (the outputs equal the states for these models)."""
        return getattr(self, "sampled_trajectories_", [])

    def getSampledCostTrajectories(self):
        """Running cost of every step of each re-rolled sample."""
        return getattr(self, "sampled_costs_", [])

    def getSampledCrashStatus(self):
        """Crash flag after every step of each re-rolled sample (crash_status_d of visualizeKernel)."""
        return getattr(self, "sampled_crash_status_", [])

    def getTopTransformedCosts(self):
        """Weights of the top-N samples divided by the normaliser."""
        return getattr(self, "top_n_costs_", np.empty(0, np.float32))

    def getFreeEnergyStatistics(self, ind=0):
        out = np.empty(6, dtype=np.float32)
        A.call("mppi_get_free_energy", self._h, int(ind), _fptr(out))
        keys = ("freeEnergyMean", "freeEnergyVariance", "freeEnergyModifiedVariance", "normalizerPercent",
                "increase", "previousBaseline")
        return dict(zip(keys, map(float, out)))

    # ---- parameters
    def getParams(self):
        return self.params_

    def setParams(self, params: A.ControllerParams):
        A.call("mppi_set_controller_params", self._h, C.byref(params))
        self.params_ = params

    def setSamplingParams(self, sampler):
        sp = sampler.to_c()
        A.call("mppi_set_sampling_params", self._h, C.byref(sp))
        self.sampler_ = sampler

    def updateDynamicsParams(self, model):
        """Dynamics::setParams of every instance (the plugin's current parameters)."""
        p = model.getParams()
        arr = (type(p) * self.num_instances)(*([p] * self.num_instances))
        A.call("mppi_set_dynamics_params", self._h, C.cast(arr, C.c_void_p), C.sizeof(arr))
        self._dyn_arr = arr

    def updateCostParams(self, cost):
        """Cost::setParams of every instance (the plugin's current parameters)."""
        p = cost.getParams()
        arr = (type(p) * self.num_instances)(*([p] * self.num_instances))
        A.call("mppi_set_cost_params", self._h, C.cast(arr, C.c_void_p), C.sizeof(arr))
        self._cost_arr = arr

    def getDt(self) -> float:
        """Controller::getDt."""
        return float(self.params_.dt)

    def getNumTimesteps(self) -> int:
        """Controller::getNumTimesteps (the longest horizon of the handle)."""
        return int(self.T.max())

    def setCostmap(self, costmap, resolution=0.1, origin=(0.0, 0.0)):
        m = np.ascontiguousarray(costmap, dtype=np.float32)
        A.call("mppi_set_costmap", self._h, _fptr(m), int(m.shape[1]), int(m.shape[0]), float(resolution),
               float(origin[0]), float(origin[1]))

    def setMLP(self, params, precision="bf16"):
        """Load surrogate weights (MPPI_MLP_PARAMS floats) into the MLP dynamics; precision "bf16" or "fp8"."""
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(-1))
        prec = BicycleSlipMLPDynamics.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        A.call("mppi_set_mlp", self._h, _fptr(p), p.size, prec)

    def setJudge(self, fraction=0.01):
        """Re-roll the ceil(fraction * K) lowest-cost surrogate samples with the analytic model (0 disables)."""
        A.call("mppi_set_judge", self._h, float(fraction))

    def judgeStats(self):
        """Per instance (mean(analytic - surrogate) cost, mean relative |analytic - surrogate|) over judged samples."""
        out = np.empty(2 * self.num_instances, dtype=np.float32)
        A.call("mppi_get_judge_stats", self._h, _fptr(out))
        return out.reshape(-1, 2)

    def useAnalyticDynamics(self, enable=True):
        """Fallback of the surrogate model: roll out the analytic dynamics instead of the network."""
        A.call("mppi_use_analytic_dynamics", self._h, int(bool(enable)))

    def injectNoise(self, noise):
        """Parity hook: use this standard-normal noise (all instances, samples layout) instead of Philox noise."""
        if noise is None:
            A.call("mppi_inject_noise", self._h, None, 0)
            return
        n = np.ascontiguousarray(np.asarray(noise, dtype=np.float32).reshape(-1))
        A.call("mppi_inject_noise", self._h, _fptr(n), n.size)
        self._injected = n

    def generateSamples(self, optimization_stride=1, iteration_num=0):
        A.call("mppi_generate_samples", self._h, int(optimization_stride), int(iteration_num))

    def setGraphMode(self, enable: bool):
        A.call("mppi_set_graph_mode", self._h, int(bool(enable)))

    def autotune(self, cache_path=None):
        A.call("mppi_autotune", self._h, None if cache_path is None else str(cache_path).encode())

    def setRolloutMode(self, mode):
        """0 = fused rollout kernel, 1 = split dynamics / cost kernels, 2 = cooperative (four lanes per sample),
        3 = sampler kernel then the staged rollout, 4 = fused with noise warps; modes 1, 2 and 4 are for small
        problems; samples and costs are bit-identical."""
        A.call("mppi_set_rollout_mode", self._h, int(mode))

    def rolloutMode(self):
        """(current mode, bitmask of available modes)."""
        m, av = C.c_int(), C.c_int()
        A.call("mppi_get_rollout_mode", self._h, C.byref(m), C.byref(av))
        return m.value, av.value

    def launchConfig(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        A.call("mppi_get_launch_config", self._h, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def setLaunchConfig(self, rollout_samples_per_cta, reduction_samples_per_cta):
        A.call("mppi_set_launch_config", self._h, int(rollout_samples_per_cta), 0, int(reduction_samples_per_cta))

    def kernelsPerCompute(self) -> int:
        n = C.c_int()
        A.call("mppi_kernels_per_compute", self._h, C.byref(n))
        return n.value

    def enqueueSolve(self, optimization_stride=1, count=1):
        """Device-resident solves with no host round trip (see mppi_enqueue_solve)."""
        A.call("mppi_enqueue_solve", self._h, int(optimization_stride), int(count))

    def synchronize(self):
        A.call("mppi_synchronize", self._h)

    def timeKernels(self, optimization_stride=1, reps=10):
        """Average device ms per launch of (sampler, rollout, weights+update)."""
        out = np.zeros(3, dtype=np.float32)
        A.call("mppi_time_kernels", self._h, int(optimization_stride), int(reps), _fptr(out))
        return out

    def stream(self) -> int:
        return A.lib().mppi_get_stream(self._h) or 0

    # ---- ancillary feedback controller (Controller's feedback methods, controller.cuh:265-269,354-414,455-571,730-743)
    def _attach_feedback(self, fb_controller):
        self.fb_controller_ = fb_controller
        self._fb_prop = None
        if fb_controller is not None:
            fb_controller._controllers.append(self)
            self.setFeedbackParams(fb_controller.params_)

    def setFeedbackParams(self, params: DDPParams):
        """Controller::setFeedbackParams (controller.cuh:735-738)."""
        S, Cd = self.S, self.Cdim
        q, qf, r = _col_major(params.Q, S), _col_major(params.Q_f, S), _col_major(params.R, Cd)
        A.call("mppi_set_feedback_params", self._h, None if q is None else _fptr(q),
               None if qf is None else _fptr(qf), None if r is None else _fptr(r), int(params.num_iterations))
        self._fb_params = params

    def getFeedbackParams(self) -> DDPParams:
        return getattr(self, "_fb_params", DDPParams())

    def initFeedback(self):
        """Controller::initFeedback: feedback on, gains reset to zero."""
        A.call("mppi_enable_feedback", self._h, 1)
        self._fb_enabled = True

    def disableFeedbackController(self):
        A.call("mppi_enable_feedback", self._h, 0)
        self._fb_enabled = False

    def getFeedbackEnabled(self) -> bool:
        """Kept on this object as well, so that getCurrentControl (a plant's state-estimator thread) does not enter
        the handle while another thread optimises."""
        return getattr(self, "_fb_enabled", False)

    def computeFeedback(self, state):
        """Controller::computeFeedback(state): DDP from `state` around the nominal trajectory of the last solve."""
        x = np.ascontiguousarray(np.asarray(state, dtype=np.float32).reshape(-1))
        if x.size != self.S:
            raise ValueError(f"state must hold {self.S} floats")
        A.call("mppi_compute_feedback", self._h, _fptr(x))

    def _fb_T(self) -> int:
        return int(self.T[1] if self.params_.controller == A.CONTROLLER_TUBE else self.T[0])

    def getFeedbackState(self) -> DDPFeedbackState:
        """Controller::getFeedbackState: a copy of the current gain trajectory."""
        g = np.empty(self._fb_T() * self.Cdim * self.S, dtype=np.float32)
        A.call("mppi_get_feedback_gains", self._h, _fptr(g))
        return DDPFeedbackState(g, self.S, self.Cdim)

    def getFeedbackControl(self, state, goal_state, t):
        """Controller::getFeedbackControl: K_t (state - goal_state)."""
        x = np.ascontiguousarray(np.asarray(state, dtype=np.float32).reshape(-1))
        g = np.ascontiguousarray(np.asarray(goal_state, dtype=np.float32).reshape(-1))
        if x.size != self.S or g.size != self.S:
            raise ValueError(f"state and goal_state must hold {self.S} floats")
        out = np.empty(self.Cdim, dtype=np.float32)
        A.call("mppi_get_feedback_control", self._h, _fptr(x), _fptr(g), int(t), _fptr(out))
        return out

    def computeFeedbackPropagatedStateSeq(self):
        """Controller::computeFeedbackPropagatedStateSeq: the state trajectory under nominal control plus feedback."""
        out = np.empty(self._fb_T() * self.S, dtype=np.float32)
        A.call("mppi_get_feedback_propagated_state_seq", self._h, _fptr(out))
        self._fb_prop = out.reshape(-1, self.S).T.copy()

    def getFeedbackPropagatedStateSeq(self) -> np.ndarray:
        if getattr(self, "_fb_prop", None) is None:
            return np.zeros((self.S, self._fb_T()), np.float32)
        return self._fb_prop

    def _rel_index(self, rel_time, T):
        dt = self.getDt()
        lower = int(rel_time / dt)
        alpha = (rel_time - lower * dt) / dt
        # the reference reads column lower + 1 unchecked; both indices are held inside the horizon here
        return min(max(lower, 0), T - 1), min(max(lower + 1, 0), T - 1), alpha

    def interpolateControls(self, rel_time, c_traj):
        """Controller::interpolateControls (controller.cuh:384-394): linear between the bracketing steps."""
        c = np.asarray(c_traj, dtype=np.float32)
        lo, hi, a = self._rel_index(rel_time, c.shape[1])
        return ((1.0 - a) * c[:, lo] + a * c[:, hi]).astype(np.float32)

    def interpolateState(self, s_traj, rel_time):
        """Controller::interpolateState (controller.cuh:396-403) with Dynamics::interpolateState (linear)."""
        s = np.asarray(s_traj, dtype=np.float32)
        lo, hi, a = self._rel_index(rel_time, s.shape[1])
        return ((1.0 - a) * s[:, lo] + a * s[:, hi]).astype(np.float32)

    def interpolateFeedback(self, state, target_nominal_state, rel_time, fb_state: DDPFeedbackState):
        """FeedbackController::interpolateFeedback_ (feedback.cuh:216-228): the gains of the bracketing steps,
        blended linearly, applied to state - target_nominal_state."""
        e = np.asarray(state, np.float32).reshape(-1) - np.asarray(target_nominal_state, np.float32).reshape(-1)
        T = fb_state.fb_gain_traj_.size // (self.S * self.Cdim)
        lo, hi, a = self._rel_index(rel_time, T)
        return ((1.0 - a) * (fb_state.gain(lo) @ e) + a * (fb_state.gain(hi) @ e)).astype(np.float32)

    def enforceConstraints(self, u):
        """Dynamics::enforceConstraints (dynamics.cu:107-126) with the handle's constraints: deadband, then clamp."""
        cc = self.constraints_
        out = np.array(u, dtype=np.float32).reshape(-1)
        for i in range(out.size):
            db = np.float32(cc.deadband[i])
            if abs(out[i]) < db:
                out[i] = np.float32(cc.zero_control[i])
            else:
                out[i] = out[i] + db * -np.sign(out[i])
            out[i] = min(max(np.float32(cc.lower[i]), out[i]), np.float32(cc.upper[i]))
        return out

    def getCurrentControl(self, state, rel_time, target_nominal_state, c_traj, fb_state=None):
        """Controller::getCurrentControl (controller.cuh:347-362): the nominal control at rel_time plus, with feedback
        on, the interpolated feedback against target_nominal_state, then the constraints with a zero state."""
        u = self.interpolateControls(rel_time, c_traj)
        if fb_state is not None and self.getFeedbackEnabled():
            u = u + self.interpolateFeedback(state, target_nominal_state, rel_time, fb_state)
        return self.enforceConstraints(u)


class VanillaMPPIController(BatchedMPPIController):
    """VanillaMPPIController(model, cost, fb_controller, sampler, dt, max_iter, lambda, alpha, num_timesteps,
    init_control_traj, stream) (controllers/MPPI/mppi_controller.cu:16-29), one instance with NUM_ROLLOUTS samples."""

    def __init__(self, model, cost, fb_controller, sampler, dt, max_iter, lambda_, alpha, num_timesteps,
                 num_rollouts, init_control_traj=None, stream=0, seed=0, slide_control_scale=None):
        init = None
        if init_control_traj is not None:
            init = np.asarray(init_control_traj, dtype=np.float32).reshape(model.CONTROL_DIM, num_timesteps).T
        super().__init__(model, cost, sampler, [num_rollouts], [num_timesteps], dt=dt, max_iter=max_iter,
                         lambda_=lambda_, alpha=alpha, seed=seed, init_control_traj=init, stream=stream,
                         slide_control_scale=slide_control_scale)
        # the feedback controller's parameters go to the handle; feedback stays off until initFeedback()
        self._attach_feedback(fb_controller)

    def getControlSeq(self) -> np.ndarray:
        return self.getControlSeqs()[0]

    def setControlSeq(self, seq):
        self.setControlSeqs([seq])

    def getTargetStateSeq(self) -> np.ndarray:
        return self.getTargetStateSeqs()[0]

    def getSampledCostSeq(self) -> np.ndarray:
        """The exp-weights the reference's trajectory_costs_ holds after an iteration (controller.cuh:449-452)."""
        return self.sample_weights()

    def getNormalizerPercent(self) -> float:
        return self.getNormalizerCost() / float(self.K[0])


class ColoredMPPIController(VanillaMPPIController):
    """ColoredMPPIController(model, cost, fb_controller, sampler, dt, max_iter, lambda, alpha, num_timesteps, ...)
    (controllers/ColoredMPPI/colored_mppi_controller.cuh:40-196): the same iteration with Tsallis weights
    (TsallisTransform, mppi_common.cu:1004-1021) once gamma and r are both non-zero, an optional state leash
    (Dynamics::enforceLeash) and, after smoothing, a clamp of control 1 only (colored_mppi_controller.cu:224-229).
    ColoredMPPIParams' defaults: r = 2, gamma = 0 (exponential weights), leash off."""

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        cp = self.getParams()
        cp.controller = A.CONTROLLER_COLORED
        self.setParams(cp)

    def _update(self, **fields):
        cp = self.getParams()
        for k, v in fields.items():
            setattr(cp, k, v)
        self.setParams(cp)

    def setGamma(self, gamma):
        self._update(tsallis_gamma=float(gamma))

    def getGamma(self) -> float:
        return float(self.params_.tsallis_gamma)

    def setRExp(self, r):
        self._update(tsallis_r=float(r))

    def getRExp(self) -> float:
        return float(self.params_.tsallis_r)

    def setStateLeashLength(self, new_state_leash, index=0):
        cp = self.getParams()
        cp.state_leash_dist[index] = float(new_state_leash)
        self.setParams(cp)

    def getStateLeashLength(self, index) -> float:
        return float(self.params_.state_leash_dist[index])

    def setLeashActive(self, active):
        self._update(leash_active=int(bool(active)))

    def getLeashActive(self) -> bool:
        return bool(self.params_.leash_active)

    def setOffsetDecayRate(self, rate):
        self.sampler_.offset_decay_rate = float(rate)
        self.setSamplingParams(self.sampler_)

    def getOffsetDecayRate(self) -> float:
        return float(self.sampler_.offset_decay_rate)

    def setColoredNoiseExponents(self, exponents):
        self.sampler_.exponents = tuple(float(v) for v in exponents)
        self.setSamplingParams(self.sampler_)

    def getColoredNoiseExponents(self):
        return list(self.sampler_.exponents)[:self.Cdim]

    def setNoiseDecay(self, decay):
        self.sampler_.std_dev_decay = float(decay)
        self.setSamplingParams(self.sampler_)


class TubeMPPIController(BatchedMPPIController):
    """TubeMPPIController(model, cost, fb_controller, sampler, dt, max_iter, lambda, alpha, num_timesteps,
    num_rollouts, ...) (controllers/Tube-MPPI/tube_mppi_controller.cuh:29-141): two sampling distributions of
    num_rollouts samples each, the actual system (instance 0, rolled out from the state given to computeControl) and
    the nominal system (instance 1, from the nominal state the controller keeps); the nominal pair takes over the
    actual pair's sequences when the actual baseline beats the nominal one by nominal_threshold.  getControlSeq and
    getTargetStateSeq are the nominal system's, as in the reference; the ancillary feedback controller (a
    DDPFeedback, or identity weights when fb_controller is None) tracks it and is on from construction."""

    def __init__(self, model, cost, fb_controller, sampler, dt, max_iter, lambda_, alpha, num_timesteps,
                 num_rollouts, init_control_traj=None, stream=0, seed=0, nominal_threshold=20.0):
        init = None
        if init_control_traj is not None:
            one = np.asarray(init_control_traj, dtype=np.float32).reshape(model.CONTROL_DIM, num_timesteps).T
            init = np.concatenate([one.reshape(-1), one.reshape(-1)])
        super().__init__(model, cost, sampler, [num_rollouts] * 2, [num_timesteps] * 2, dt=dt, max_iter=max_iter,
                         lambda_=lambda_, alpha=alpha, seed=seed, init_control_traj=init, stream=stream)
        cp = self.getParams()
        cp.controller = A.CONTROLLER_TUBE
        cp.nominal_threshold = float(nominal_threshold)
        self.setParams(cp)
        # Tube-MPPI runs its ancillary controller from the start (tube_mppi_controller.cu:27-29)
        self._attach_feedback(fb_controller)
        self.initFeedback()

    def computeControl(self, state, optimization_stride=1):
        """TubeMPPIController::computeControl (tube_mppi_controller.cu:158-296); state: the actual system's."""
        x = np.ascontiguousarray(np.asarray(state, dtype=np.float32).reshape(-1))
        if x.size != self.S:
            raise ValueError(f"state must hold {self.S} floats")
        A.call("mppi_compute_control", self._h, _fptr(x), int(optimization_stride))

    def getControlSeq(self) -> np.ndarray:
        """The nominal control sequence (TubeMPPIController::getControlSeq, tube_mppi_controller.cuh:61-64)."""
        return self.getControlSeqs()[1]

    def getNominalControlSeq(self) -> np.ndarray:
        return self.getControlSeqs()[1]

    def getActualControlSeq(self) -> np.ndarray:
        """The actual system's control sequence (TubeMPPIController::getActualControlSeq, :77-80)."""
        return self.getControlSeqs()[0]

    def setControlSeq(self, seq):
        s = np.asarray(seq, np.float32)
        self.setControlSeqs([s, s])

    def getTargetStateSeq(self) -> np.ndarray:
        """The nominal state trajectory (TubeMPPIController::getTargetStateSeq, tube_mppi_controller.cuh:69-72)."""
        return self.getTargetStateSeqs()[1]

    def getNominalStateSeq(self) -> np.ndarray:
        return self.getTargetStateSeqs()[1]

    def getActualStateSeq(self) -> np.ndarray:
        """The actual system's state trajectory (Controller::getActualStateSeq, controller.cuh:538-541)."""
        return self.getTargetStateSeqs()[0]

    def getNominalThreshold(self) -> float:
        return float(self.params_.nominal_threshold)

    def setNominalThreshold(self, threshold):
        cp = self.getParams()
        cp.nominal_threshold = float(threshold)
        self.setParams(cp)

    def nominalStateUsed(self) -> int:
        """FreeEnergyStatistics::nominal_state_used of the last computeControl."""
        v = C.c_int()
        A.call("mppi_get_nominal_state_used", self._h, C.byref(v))
        return v.value


class RobustMPPIController(BatchedMPPIController):
    """RobustMPPIController(model, cost, fb_controller, sampler, dt, max_iter, lambda, alpha, value_function_threshold,
    num_timesteps, num_rollouts, init_control_traj, num_candidate_nominal_states, optimization_stride, ...)
    (controllers/R-MPPI/robust_mppi_controller.cu:12-45): two sampling distributions of num_rollouts samples in the
    reference's order, the nominal system (instance 0, from the nominal state) and the real system (instance 1, from
    the state given to computeControl, its controls corrected by the DDP feedback against the nominal state), both
    around the nominal sequence.  updateImportanceSamplingControl(state, stride) chooses the nominal state among
    candidates between the nominal trajectory and the real state, slides the nominal sequence and computes the
    feedback gains; call it before each computeControl.  getControlSeq is the real system's sequence and
    getTargetStateSeq the nominal state trajectory, as in the reference; slideControlSequence and computeFeedback do
    nothing (the importance-sampler update does both).  Analytic models with Gaussian sampling: the built-in ones here,
    a caller's plugin pair through plugin.PluginRobustMPPIController."""

    def __init__(self, model, cost, fb_controller, sampler, dt, max_iter, lambda_, alpha, value_function_threshold,
                 num_timesteps, num_rollouts, init_control_traj=None, num_candidate_nominal_states=9,
                 optimization_stride=1, num_eval_samples_per_candidate=64, stream=0, seed=0):
        init = None
        if init_control_traj is not None:
            one = np.asarray(init_control_traj, dtype=np.float32).reshape(model.CONTROL_DIM, num_timesteps).T
            init = np.concatenate([one.reshape(-1), one.reshape(-1)])
        super().__init__(model, cost, sampler, [num_rollouts] * 2, [num_timesteps] * 2, dt=dt, max_iter=max_iter,
                         lambda_=lambda_, alpha=alpha, seed=seed, init_control_traj=init, stream=stream)
        cp = self.getParams()
        cp.controller = A.CONTROLLER_RMPPI
        cp.value_function_threshold = float(value_function_threshold)
        cp.num_candidate_nominal_states = int(num_candidate_nominal_states)
        cp.num_eval_samples_per_candidate = int(num_eval_samples_per_candidate)
        self.setParams(cp)
        self.optimization_stride_ = int(optimization_stride)
        # the constructor turns the feedback on (robust_mppi_controller.cu:37-43)
        self._attach_feedback(fb_controller)
        self._fb_enabled = True

    def updateImportanceSamplingControl(self, state, stride=1):
        """RobustMPPIController::updateImportanceSamplingControl (robust_mppi_controller.cu:548-569)."""
        x = np.ascontiguousarray(np.asarray(state, dtype=np.float32).reshape(-1))
        if x.size != self.S:
            raise ValueError(f"state must hold {self.S} floats")
        A.call("mppi_rmppi_update_importance_sampler", self._h, _fptr(x), int(stride))

    def computeControl(self, state, optimization_stride=1):
        """RobustMPPIController::computeControl (robust_mppi_controller.cu:635-744); state: the real system's."""
        x = np.ascontiguousarray(np.asarray(state, dtype=np.float32).reshape(-1))
        if x.size != self.S:
            raise ValueError(f"state must hold {self.S} floats")
        A.call("mppi_compute_control", self._h, _fptr(x), int(optimization_stride))

    def getControlSeq(self) -> np.ndarray:
        """The real system's sequence (RobustMPPIController::getControlSeq, robust_mppi_controller.cuh:136-139)."""
        return self.getControlSeqs()[1]

    def getNominalControlSeq(self) -> np.ndarray:
        return self.getControlSeqs()[0]

    def setControlSeq(self, seq):
        s = np.asarray(seq, np.float32)
        self.setControlSeqs([s, s])

    def getTargetStateSeq(self) -> np.ndarray:
        """The nominal state trajectory (RobustMPPIController::getTargetStateSeq, :141-144)."""
        return self.getTargetStateSeqs()[0]

    def getActualStateSeq(self) -> np.ndarray:
        """The real system's state trajectory under its sequence, from the state of the last computeControl."""
        return self.getTargetStateSeqs()[1]

    def _candidates(self):
        cp = self.params_
        N, J = int(cp.num_candidate_nominal_states), int(cp.num_eval_samples_per_candidate)
        best, stride = C.c_int(), C.c_int()
        states = np.zeros(N * self.S, np.float32)
        strides = np.zeros(N, np.int32)
        fe = np.zeros(N, np.float32)
        costs = np.zeros(N * J, np.float32)
        A.call("mppi_rmppi_get_candidates", self._h, C.byref(best), C.byref(stride), _fptr(states),
               strides.ctypes.data_as(C.POINTER(C.c_int)), _fptr(fe), _fptr(costs))
        return best.value, stride.value, states.reshape(N, self.S), strides, fe, costs

    def getNominalState(self) -> np.ndarray:
        """RobustMPPIController::getNominalState: the nominal system's initial state."""
        return self.getTargetStateSeq()[:, 0].copy()

    def getBestIndex(self) -> int:
        return self._candidates()[0]

    def getNominalStride(self) -> int:
        return self._candidates()[1]

    def getCandidateStates(self) -> np.ndarray:
        return self._candidates()[2]

    def getCandidateStrides(self) -> np.ndarray:
        return self._candidates()[3]

    def getCandidateFreeEnergy(self) -> np.ndarray:
        return self._candidates()[4]

    def getCandidateEvalCosts(self) -> np.ndarray:
        return self._candidates()[5]

    def getValueFunctionThreshold(self) -> float:
        return float(self.params_.value_function_threshold)

    def getNumCandidates(self) -> int:
        return int(self.params_.num_candidate_nominal_states)

    def getNumEvalSamplesPerCandidate(self) -> int:
        return int(self.params_.num_eval_samples_per_candidate)

    def getOptimizationStride(self) -> int:
        return self.optimization_stride_
