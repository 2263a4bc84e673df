"""Kinematic bicycle on a costmap and the 7-state dynamic bicycle: computeControl parity with the oracle given
injected noise.  Trig, bilinear costmap lookups and Euler steps use the same float arithmetic on both sides, so the
per-sample costs are bit-identical; the FP64 oracle measures the float rollout's accuracy."""
import numpy as np
import pytest

import _parity
import oracle
from mppi_generic_vendor_gb300 import (BicycleDynamics, BicycleSlipDynamics, CostmapCost, GaussianDistribution,
                                       VanillaMPPIController)
from mppi_generic_vendor_gb300 import _abi as A
from mppi_generic_vendor_gb300.workloads import gaussian_bump_costmap

pytestmark = pytest.mark.gpu


def run_parity(dyn, x0, std, lam, K, T, seed, map_size=128):
    cmap = gaussian_bump_costmap(seed, size=map_size)
    cost = CostmapCost(map_coeff=1.0, speed_target=8.0, speed_coeff=1.0, steer_coeff=0.5, terminal_coeff=2.0,
                       costmap=cmap, resolution=0.1, origin=(0.0, 0.0))
    ctrl = VanillaMPPIController(dyn, cost, None, GaussianDistribution(std_dev=std), 0.02, 1, lam, 0.0, T, K)
    rng = np.random.default_rng(seed)
    Cd = dyn.CONTROL_DIM
    eps = rng.standard_normal(K * T * Cd).astype(np.float32)
    init = rng.uniform(-0.2, 0.2, (T, Cd)).astype(np.float32)
    ctrl.setControlSeq(init.T)
    ctrl.injectNoise(eps)
    ctrl.computeControl(x0, 1)
    ref = oracle.compute_control(ctrl.model_id, ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.getParams(),
                                 ctrl.sampler_.to_c(), ctrl.constraints_, K, T, Cd, dyn.STATE_DIM, x0, eps, init,
                                 costmap=(cmap, 0.1, (0.0, 0.0)))
    got = ctrl.sample_costs()
    assert np.array_equal(got.view(np.uint32), ref["costs"].view(np.uint32))
    assert ctrl.getBaselineCost() == ref["baseline"]
    _parity.check_control(ctrl.getControlSeq().T, ref, K, T, Cd)
    # accuracy of the float rollout against FP64 (same constrained samples)
    sp = ctrl.sampler_.to_c()
    r64, _, _ = oracle.rollout(ctrl.model_id, ctrl._dyn_arr[0], ctrl._cost_arr[0], x0, ref["samples"], init, sp,
                               ctrl.constraints_, lam, 0.0, K, T, 0.02, costmap=(cmap, 0.1, (0.0, 0.0)), fp64=True,
                               state_dim=dyn.STATE_DIM)
    rel = np.abs(got - r64) / np.abs(r64)
    ctrl.close()
    return rel


def test_bicycle_costmap_parity():
    dyn = BicycleDynamics(2.5)
    x0 = np.array([6.0, 5.0, 0.4, 4.0], np.float32)
    rel = run_parity(dyn, x0, (1.0, 0.3), 2.0, 2048, 100, 3)
    assert np.median(rel) < 1e-5


def test_bicycle_costmap_parity_benchmark_size():
    """The kinematic-bicycle benchmark configuration itself: K = 16384, T = 100, the 512 x 512 costmap of 32 bumps at
    0.1 m cells, sigma (1.0, 0.3), lambda 2.0."""
    dyn = BicycleDynamics(2.5)
    dyn.setControlRanges([(-3.0, 3.0), (-1.0, 1.0)])
    x0 = np.array([25.0, 25.0, 0.3, 4.0], np.float32)
    rel = run_parity(dyn, x0, (1.0, 0.3), 2.0, 16384, 100, 0, map_size=512)
    assert np.median(rel) < 1e-5


def test_bicycle_slip_parity():
    dyn = BicycleSlipDynamics()
    x0 = np.array([6.0, 5.0, 0.2, 6.0, 0.0, 0.0, 0.0], np.float32)
    rel = run_parity(dyn, x0, (0.5, 0.5), 2.0, 1024, 60, 4)
    assert np.median(rel) < 1e-4


def test_costmap_required():
    dyn = BicycleDynamics(2.5)
    cost = CostmapCost()
    ctrl = VanillaMPPIController(dyn, cost, None, GaussianDistribution(std_dev=(1.0, 0.3)), 0.02, 1, 2.0, 0.0, 20, 64)
    with pytest.raises(A.MPPIError):
        ctrl.computeControl(np.zeros(4, np.float32))
    ctrl.close()
