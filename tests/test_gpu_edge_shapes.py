"""Edge shapes against the oracle: a single sample, a single step, horizons whose sample rows are not whole 16-byte
quads, sample counts one off the rollout tile sizes, in every rollout mode the shape allows and at the smallest and
largest rollout tile (32 and 256 samples per CTA).  Per-sample costs and constrained samples bit-identical, baseline
exact, the update element-wise within 1e-5 of its term magnitude (the same criterion as the full-size tests)."""
import numpy as np
import pytest

import _parity
import oracle
from mppi_generic_vendor_gb300 import (BicycleDynamics, BicycleSlipDynamics, CartpoleDynamics, CartpoleSwingupCost,
                                       CostmapCost, DoubleIntegratorDynamics, DoubleIntegratorObstacleCost,
                                       GaussianDistribution, VanillaMPPIController)
from mppi_generic_vendor_gb300.workloads import gaussian_bump_costmap

pytestmark = pytest.mark.gpu

# (K, T): one sample and one step; rows of 1, 3, 6, 9 steps (C = 1: never a whole quad; C = 2: a quad for even T);
# K one below / above the 32, 64 and 128-sample tiles
SHAPES = [(1, 1), (1, 6), (2, 1), (7, 3), (31, 4), (33, 9), (65, 2), (129, 8)]
MODES = ["cartpole", "double_integrator", "bicycle_costmap", "bicycle_slip"]


def _model(name, rng):
    """(dynamics, cost, x0, std, costmap or None) of each built-in model."""
    if name == "cartpole":
        dyn = CartpoleDynamics(1.0, 1.0, 1.0)
        dyn.setControlRanges([(-5.0, 5.0)])
        cost = CartpoleSwingupCost(10.0, 1.0, 100.0, 1.0, 0.0)
        x0 = np.array([0.05, -0.02, rng.uniform(-np.pi, np.pi), 0.03], np.float32)
        return dyn, cost, x0, (1.0,), None
    if name == "double_integrator":
        dyn = DoubleIntegratorDynamics()
        dyn.setControlRanges([(-1.0, 1.0), (-1.0, 1.0)])
        obs = [(rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(0.3, 1.0)) for _ in range(8)]
        cost = DoubleIntegratorObstacleCost(goal=(1.5, -1.0, 0.0, 0.0), coeff=(1.0, 1.0, 0.1, 0.1), terminal_coeff=10.0,
                                            obstacles=obs, obstacle_cost=1000.0)
        return dyn, cost, rng.uniform(-2, 2, 4).astype(np.float32), (0.5, 0.5), None
    cmap = gaussian_bump_costmap(5, size=128)
    cost = CostmapCost(map_coeff=1.0, speed_target=8.0, speed_coeff=1.0, steer_coeff=0.5, terminal_coeff=2.0,
                       costmap=cmap, resolution=0.1, origin=(0.0, 0.0))
    if name == "bicycle_costmap":
        dyn = BicycleDynamics(2.5)
        dyn.setControlRanges([(-3.0, 3.0), (-1.0, 1.0)])
        return dyn, cost, np.array([6.0, 5.0, 0.4, 4.0], np.float32), (1.0, 0.3), cmap
    dyn = BicycleSlipDynamics()
    return dyn, cost, np.array([6.0, 5.0, 0.2, 6.0, 0.1, 0.0, 0.0], np.float32), (0.5, 0.5), cmap


@pytest.mark.parametrize("K,T", SHAPES)
@pytest.mark.parametrize("name", MODES)
def test_edge_shape_parity_in_every_rollout_mode(name, K, T):
    rng = np.random.default_rng(K * 1000 + T)
    dyn, cost, x0, std, cmap = _model(name, rng)
    Cd, S = dyn.CONTROL_DIM, dyn.STATE_DIM
    ctrl = VanillaMPPIController(dyn, cost, None, GaussianDistribution(std_dev=std), 0.02, 1, 1.5, 0.0, T, K)
    eps = rng.standard_normal(K * T * Cd).astype(np.float32)
    init = rng.uniform(-0.3, 0.3, (T, Cd)).astype(np.float32)
    extra = {} if cmap is None else {"costmap": (cmap, 0.1, (0.0, 0.0))}
    ref = oracle.compute_control(ctrl.model_id, ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.getParams(),
                                 ctrl.sampler_.to_c(), ctrl.constraints_, K, T, Cd, S, x0, eps, init, **extra)
    _, avail = ctrl.rolloutMode()
    ran = 0
    for mode in range(5):
        if not (avail >> mode) & 1:
            continue
        for ns in (32, 256):
            ctrl.setRolloutMode(mode)
            ctrl.setLaunchConfig(ns, 256)
            ctrl.setControlSeq(init.T)
            ctrl.injectNoise(eps)
            ctrl.computeControl(x0, 1)
            where = (name, K, T, mode, ns)
            assert np.array_equal(ctrl.sample_costs().view(np.uint32), ref["costs"].view(np.uint32)), where
            assert np.array_equal(ctrl.control_samples().view(np.uint32), ref["samples"].view(np.uint32)), where
            assert ctrl.getBaselineCost() == ref["baseline"], where
            _parity.check_control(ctrl.getControlSeq().T, ref, K, T, Cd)
            ran += 1
    assert ran >= 2  # mode 0 at both tile sizes at least
    ctrl.close()
