"""Seeded synthetic workloads with the shapes of the benchmark configurations.

* ``cartpole``   — plain MPPI, cartpole, K=2048, T=100, sigma 1.0, lambda 1.0, force clamped to +-5 N, dt 0.02,
  x0 with theta ~ U(-pi, pi) and the other states ~ U(-0.1, 0.1), receding horizon.
* ``batched_di`` — 256 double-integrator instances, K ~ U{512, 1024, 2048, 4096, 8192}, T ~ U{32, 64, 128},
  controls clamped to +-1, colored noise with exponents (1, 1) and sigma 0.5, goal + 8 circular obstacles
  (centres U(-5, 5)^2, radii U(0.3, 1.0), cost 1000 inside).
* ``bicycle``    — kinematic bicycle on a 512x512 costmap (0.1 m cells) built from 32 Gaussian bumps
  (amplitude U(0, 10), sigma U(0.5, 3) m), speed target 8 m/s, K=16384, T=100, sigma (1.0, 0.3), lambda 2.0.
* ``slip_mlp``   — the 7-state dynamic bicycle through the learned 9-64-64-5 surrogate (trained on the GPU on 2^20
  transitions of the analytic model), BF16 weights, K=16384, T=100, analytic judge on the top 1% of samples, the
  costmap of ``bicycle``, sigma (0.5, 0.5), lambda 2.0.
* ``batched_slip_mlp`` — 128 surrogate instances with K ~ U[2048, 16384] and T ~ U{50, 100, 200}, FP8 E4M3 weights
  with one scale per layer, one shared costmap as in ``bicycle``.
* ``cartpole_rmppi`` — the robust controller (R-MPPI) on the cart-pole of ``cartpole``: two distributions of K=2048
  samples, T=100, 9 candidate nominal states with 64 evaluation samples each, value-function threshold 1000, the DDP
  feedback with identity weights; one iteration = the importance-sampler update + the solve.
* ``cartpole_tube`` — Tube-MPPI on the same cart-pole: two distributions of K=2048 samples, T=100, nominal threshold
  20, the DDP feedback with identity weights; one iteration = the solve + the feedback gains + a one-step slide.

There is no public dataset behind these configurations; every input is drawn from a recorded seed.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .controller import (BatchedMPPIController, BicycleDynamics, BicycleSlipMLPDynamics, CartpoleDynamics,
                         CartpoleSwingupCost,
                         ColoredNoiseDistribution, CostmapCost, DDPFeedback, DoubleIntegratorDynamics,
                         DoubleIntegratorObstacleCost, GaussianDistribution, RobustMPPIController,
                         TubeMPPIController, VanillaMPPIController)


@dataclass
class Workload:
    name: str
    controller: BatchedMPPIController  # None for a description-only workload (describe_only=True)
    x0: np.ndarray            # float32 [num_instances * S]
    K: np.ndarray
    T: np.ndarray
    state_dim: int
    control_dim: int
    num_iters: int
    description: dict = field(default_factory=dict)
    eval_sample_steps: int = 0  # R-MPPI: the candidate evaluation's rollout steps per iteration

    @property
    def sample_steps_per_iter(self) -> int:
        return int(np.sum(self.K.astype(np.int64) * self.T)) + self.eval_sample_steps

    @property
    def control_floats(self) -> int:
        return int(np.sum(self.K.astype(np.int64) * self.T)) * self.control_dim


def cartpole(seed: int = 0, K: int = 2048, T: int = 100, stream: int = 0, describe_only: bool = False) -> Workload:
    rng = np.random.default_rng(seed)
    dyn = CartpoleDynamics(1.0, 1.0, 1.0, 9.81)
    dyn.setControlRanges([(-5.0, 5.0)])
    cost = CartpoleSwingupCost(10.0, 1.0, 100.0, 1.0, 0.0)
    ctrl = None if describe_only else VanillaMPPIController(dyn, cost, None, GaussianDistribution(std_dev=(1.0,)),
                                                            0.02, 1, 1.0, 0.0, T, K, stream=stream, seed=seed)
    x0 = np.array([rng.uniform(-0.1, 0.1), rng.uniform(-0.1, 0.1), rng.uniform(-np.pi, np.pi),
                   rng.uniform(-0.1, 0.1)], dtype=np.float32)
    return Workload("cartpole_K2048_T100", ctrl, x0, np.array([K]), np.array([T]), 4, 1, 1,
                    dict(model="cartpole", K=K, T=T, sigma=1.0, lam=1.0, dt=0.02, seed=seed))


def cartpole_rmppi(seed: int = 0, K: int = 2048, T: int = 100, num_candidates: int = 9, eval_samples: int = 64,
                   stream: int = 0, describe_only: bool = False) -> Workload:
    rng = np.random.default_rng(seed)
    dyn = CartpoleDynamics(1.0, 1.0, 1.0, 9.81)
    dyn.setControlRanges([(-5.0, 5.0)])
    cost = CartpoleSwingupCost(10.0, 1.0, 100.0, 1.0, 0.0)
    ctrl = None
    if not describe_only:
        ctrl = RobustMPPIController(dyn, cost, DDPFeedback(dyn, 0.02), GaussianDistribution(std_dev=(1.0,)), 0.02, 1,
                                    1.0, 0.0, 1000.0, T, K, num_candidate_nominal_states=num_candidates,
                                    num_eval_samples_per_candidate=eval_samples, stream=stream, seed=seed)
    x0 = np.array([rng.uniform(-0.1, 0.1), rng.uniform(-0.1, 0.1), rng.uniform(-np.pi, np.pi),
                   rng.uniform(-0.1, 0.1)], dtype=np.float32)
    return Workload(f"cartpole_rmppi_K{K}x2_T{T}", ctrl, x0, np.array([K, K]), np.array([T, T]), 4, 1, 1,
                    dict(model="cartpole", controller="R-MPPI", K=K, T=T, candidates=num_candidates,
                         eval_samples=eval_samples, threshold=1000.0, sigma=1.0, lam=1.0, dt=0.02, seed=seed),
                    eval_sample_steps=num_candidates * eval_samples * T)


def cartpole_tube(seed: int = 0, K: int = 2048, T: int = 100, stream: int = 0,
                  describe_only: bool = False) -> Workload:
    rng = np.random.default_rng(seed)
    dyn = CartpoleDynamics(1.0, 1.0, 1.0, 9.81)
    dyn.setControlRanges([(-5.0, 5.0)])
    cost = CartpoleSwingupCost(10.0, 1.0, 100.0, 1.0, 0.0)
    ctrl = None
    if not describe_only:
        ctrl = TubeMPPIController(dyn, cost, DDPFeedback(dyn, 0.02), GaussianDistribution(std_dev=(1.0,)), 0.02, 1,
                                  1.0, 0.0, T, K, stream=stream, seed=seed, nominal_threshold=20.0)
    x0 = np.array([rng.uniform(-0.1, 0.1), rng.uniform(-0.1, 0.1), rng.uniform(-np.pi, np.pi),
                   rng.uniform(-0.1, 0.1)], dtype=np.float32)
    return Workload(f"cartpole_tube_K{K}x2_T{T}", ctrl, x0, np.array([K, K]), np.array([T, T]), 4, 1, 1,
                    dict(model="cartpole", controller="Tube-MPPI", K=K, T=T, nominal_threshold=20.0, sigma=1.0,
                         lam=1.0, dt=0.02, seed=seed))


def batched_di_params(seed: int = 0, num_instances: int = 256):
    rng = np.random.default_rng(seed)
    Ks = rng.choice([512, 1024, 2048, 4096, 8192], size=num_instances)
    Ts = rng.choice([32, 64, 128], size=num_instances)
    costs, x0 = [], []
    for _ in range(num_instances):
        obs = [(rng.uniform(-5, 5), rng.uniform(-5, 5), rng.uniform(0.3, 1.0)) for _ in range(8)]
        goal = (rng.uniform(-4, 4), rng.uniform(-4, 4), 0.0, 0.0)
        costs.append(DoubleIntegratorObstacleCost(goal=goal, coeff=(1.0, 1.0, 0.1, 0.1), terminal_coeff=10.0,
                                                  obstacles=obs, obstacle_cost=1000.0))
        x0.append(np.array([rng.uniform(-5, 5), rng.uniform(-5, 5), 0.0, 0.0], dtype=np.float32))
    return Ks.astype(np.int32), Ts.astype(np.int32), costs, np.concatenate(x0)


def batched_di(seed: int = 0, num_instances: int = 256, colored: bool = True, stream: int = 0,
               describe_only: bool = False) -> Workload:
    Ks, Ts, costs, x0 = batched_di_params(seed, num_instances)
    dyn = DoubleIntegratorDynamics()
    dyn.setControlRanges([(-1.0, 1.0), (-1.0, 1.0)])
    if colored:
        sampler = ColoredNoiseDistribution(std_dev=(0.5, 0.5), exponents=(1.0, 1.0))
    else:
        sampler = GaussianDistribution(std_dev=(0.5, 0.5))
    ctrl = None if describe_only else BatchedMPPIController(dyn, costs, sampler, Ks, Ts, dt=0.02, max_iter=1,
                                                            lambda_=1.0, seed=seed, stream=stream)
    name = f"batched_di_{num_instances}x_colored" if colored else f"batched_di_{num_instances}x_gaussian"
    return Workload(name, ctrl, x0, Ks, Ts, 4, 2, 1,
                    dict(model="double_integrator", instances=num_instances, sum_K=int(Ks.sum()),
                         noise="colored beta=(1,1)" if colored else "gaussian", sigma=0.5, seed=seed))


def gaussian_bump_costmap(seed: int = 0, size: int = 512, resolution: float = 0.1, bumps: int = 32) -> np.ndarray:
    rng = np.random.default_rng(seed)
    extent = size * resolution
    c = (np.arange(size) + 0.5) * resolution
    X, Y = np.meshgrid(c, c)
    m = np.zeros((size, size), dtype=np.float64)
    for _ in range(bumps):
        a = rng.uniform(0, 10)
        s = rng.uniform(0.5, 3.0)
        cx, cy = rng.uniform(0, extent, 2)
        m += a * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s * s))
    return m.astype(np.float32)


def bicycle(seed: int = 0, K: int = 16384, T: int = 100, stream: int = 0, describe_only: bool = False) -> Workload:
    rng = np.random.default_rng(seed + 1)
    cmap = gaussian_bump_costmap(seed)
    dyn = BicycleDynamics(2.5)
    dyn.setControlRanges([(-3.0, 3.0), (-1.0, 1.0)])
    cost = CostmapCost(map_coeff=1.0, speed_target=8.0, speed_coeff=1.0, steer_coeff=0.0, terminal_coeff=0.0,
                       costmap=cmap, resolution=0.1, origin=(0.0, 0.0))
    ctrl = None if describe_only else VanillaMPPIController(dyn, cost, None, GaussianDistribution(std_dev=(1.0, 0.3)),
                                                            0.02, 1, 2.0, 0.0, T, K, stream=stream, seed=seed)
    x0 = np.array([rng.uniform(5, 45), rng.uniform(5, 45), rng.uniform(-np.pi, np.pi), 4.0], dtype=np.float32)
    return Workload("bicycle_costmap_K16384_T100", ctrl, x0, np.array([K]), np.array([T]), 4, 2, 1,
                    dict(model="bicycle_costmap", K=K, T=T, map="512x512@0.1m, 32 bumps", lam=2.0, seed=seed))


def train_surrogate(seed: int = 7, num_transitions: int = 1 << 20, steps: int | None = None, batch: int = 8192,
                    stream: int = 0, weight_format: str = "fp32", qat_steps: int = 10000) -> np.ndarray:
    """Surrogate parameters trained on the GPU by the engine's own kernels (one to three seconds on one GB300).  FP32
    weights: 10^4 Adam steps.  For a quantised deployment (weight_format "bf16" or "fp8"): 2 x 10^4 FP32 steps, then
    `qat_steps` steps of quantisation-aware fine-tuning in that format (forward and backward through the rounded
    weights), which brings MPPI on E4M3 weights from about 20% to within 1% of MPPI on the analytic model."""
    from .surrogate import Surrogate

    quantised = weight_format != "fp32" and qat_steps > 0
    s = Surrogate(num_transitions=num_transitions, seed=seed, stream=stream)
    try:
        s.generate()
        s.train(steps=steps or (20000 if quantised else 10000), batch=batch, lr=3e-3, lr_final=1e-4)
        if quantised:
            s.set_weight_format(weight_format)
            s.train(steps=qat_steps, batch=batch, lr=1e-3, lr_final=2e-5)
        return s.params()
    finally:
        s.close()


def _slip_cost(cmap):
    return CostmapCost(map_coeff=1.0, speed_target=8.0, speed_coeff=1.0, steer_coeff=0.5, terminal_coeff=2.0,
                       costmap=cmap, resolution=0.1, origin=(0.0, 0.0))


def _slip_x0(rng):
    return np.array([rng.uniform(5, 45), rng.uniform(5, 45), rng.uniform(-np.pi, np.pi), rng.uniform(4, 8), 0.0, 0.0,
                     0.0], dtype=np.float32)


def slip_mlp(seed: int = 0, K: int = 16384, T: int = 100, precision: str = "bf16", params=None, judge: float = 0.01,
             stream: int = 0, describe_only: bool = False) -> Workload:
    rng = np.random.default_rng(seed + 3)
    ctrl = None
    if not describe_only:
        if params is None:
            params = train_surrogate(stream=stream)
        dyn = BicycleSlipMLPDynamics(params, precision=precision)
        ctrl = VanillaMPPIController(dyn, _slip_cost(gaussian_bump_costmap(seed)), None,
                                     GaussianDistribution(std_dev=(0.5, 0.5)), 0.02, 1, 2.0, 0.0, T, K, stream=stream,
                                     seed=seed)
        ctrl.setJudge(judge)
    return Workload(f"slip_mlp_{precision}_K{K}_T{T}", ctrl, _slip_x0(rng), np.array([K]), np.array([T]), 7, 2, 1,
                    dict(model="bicycle_slip_mlp", precision=precision, K=K, T=T, judge=judge,
                         map="512x512@0.1m, 32 bumps", lam=2.0, seed=seed))


def batched_slip_mlp(seed: int = 0, num_instances: int = 128, precision: str = "fp8", params=None,
                     judge: float = 0.01, stream: int = 0, describe_only: bool = False) -> Workload:
    rng = np.random.default_rng(seed + 5)
    Ks = rng.integers(2048, 16385, size=num_instances).astype(np.int32)
    Ts = rng.choice([50, 100, 200], size=num_instances).astype(np.int32)
    x0 = np.concatenate([_slip_x0(rng) for _ in range(num_instances)])
    ctrl = None
    if not describe_only:
        if params is None:
            params = train_surrogate(stream=stream, weight_format=precision)
        dyn = BicycleSlipMLPDynamics(params, precision=precision)
        ctrl = BatchedMPPIController(dyn, _slip_cost(gaussian_bump_costmap(seed)),
                                     GaussianDistribution(std_dev=(0.5, 0.5)), Ks, Ts, dt=0.02, max_iter=1,
                                     lambda_=2.0, seed=seed, stream=stream)
        ctrl.setJudge(judge)
    return Workload(f"batched_slip_mlp_{num_instances}x_{precision}", ctrl, x0, Ks, Ts, 7, 2, 1,
                    dict(model="bicycle_slip_mlp", precision=precision, instances=num_instances, sum_K=int(Ks.sum()),
                         T="U{50,100,200}", judge=judge, map="512x512@0.1m, 32 bumps (shared)", lam=2.0, seed=seed))


BUILDERS = {"cartpole": cartpole, "batched_di": batched_di, "bicycle": bicycle, "slip_mlp": slip_mlp,
            "batched_slip_mlp": batched_slip_mlp}
