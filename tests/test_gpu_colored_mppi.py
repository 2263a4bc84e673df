"""ColoredMPPIController on the GPU against the oracle (colored_mppi_controller.cu:145-249).

* Tsallis weights (TsallisTransform, mppi_common.cu:1004-1021) once gamma and r are non-zero: given the same injected
  noise the per-sample costs are bit-identical, the weights agree to a few ulps scaled by the Tsallis exponent (CUDA's
  and libm's logf / expf round differently in the last place), and the updated control is within 1e-5 of its term
  magnitude (tests/_parity.py).
* gamma = 0: the exponential transform, with the controller's own final pass (only control 1 clamped).
* The state leash: the second solve starts from x0 held within the leash distances of the nominal state at the step
  the last slide moved by (Dynamics::enforceLeash, dynamics.cuh:445-463).
"""
import numpy as np
import pytest

import _parity
import oracle
from mppi_generic_vendor_gb300 import (ColoredMPPIController, DoubleIntegratorDynamics, DoubleIntegratorObstacleCost,
                                       GaussianDistribution, VanillaMPPIController)

pytestmark = pytest.mark.gpu


def _controller(cls, K, T, seed=0):
    dyn = DoubleIntegratorDynamics()
    dyn.setControlRanges([(-1.0, 1.0), (-0.5, 0.5)])
    rng = np.random.default_rng(seed)
    obs = [(rng.uniform(-5, 5), rng.uniform(-5, 5), rng.uniform(0.3, 1.0)) for _ in range(8)]
    cost = DoubleIntegratorObstacleCost(goal=(2.0, -1.0, 0.0, 0.0), coeff=(1.0, 1.0, 0.1, 0.1), terminal_coeff=10.0,
                                        obstacles=obs, obstacle_cost=1000.0)
    return cls(dyn, cost, None, GaussianDistribution(std_dev=(0.5, 0.5)), 0.02, 1, 1.0, 0.0, T, K, seed=seed)


def _solve(ctrl, K, T, rng, x0, x0_oracle=None):
    eps = rng.standard_normal(K * T * 2).astype(np.float32)
    init = rng.uniform(-0.4, 0.4, (T, 2)).astype(np.float32)
    ctrl.setControlSeq(init.T)
    ctrl.injectNoise(eps)
    ctrl.computeControl(x0, 1)
    ref = oracle.compute_control(ctrl.model_id, ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.getParams(),
                                 ctrl.sampler_.to_c(), ctrl.constraints_, K, T, 2, 4,
                                 x0 if x0_oracle is None else x0_oracle, eps, init)
    return ref


@pytest.mark.parametrize("frac,r", [(0.3, 2.0), (0.05, 1.5), (0.8, 3.0)])
def test_tsallis_weights_and_update_match_oracle(frac, r):
    """gamma is set to a fraction of the sampled cost spread, so part of the samples get weight exactly zero."""
    K, T = 4096, 64
    ctrl = _controller(ColoredMPPIController, K, T)
    x0 = np.array([-3.0, 2.0, 0.5, -0.2], np.float32)
    state = np.random.default_rng(int(100 * frac)).bit_generator.state
    rng = np.random.default_rng()
    rng.bit_generator.state = state
    _solve(ctrl, K, T, rng, x0)  # exponential weights: only to read the cost spread of these samples
    c = ctrl.sample_costs()
    gamma = float(frac * (c.max() - c.min()))
    ctrl.setGamma(gamma)
    ctrl.setRExp(r)
    rng.bit_generator.state = state  # the same noise and initial sequence again
    ref = _solve(ctrl, K, T, rng, x0)
    got = ctrl.sample_costs()
    assert np.array_equal(got.view(np.uint32), ref["costs"].view(np.uint32))
    assert ctrl.getBaselineCost() == ref["baseline"]
    w, wr = ctrl.sample_weights().astype(np.float64), ref["weights"].astype(np.float64)
    d = (ref["costs"] - ref["baseline"]).astype(np.float32)
    arg = (1.0 - (d / np.float32(gamma)).astype(np.float64)).astype(np.float32)
    expo = np.abs(np.log(np.maximum(arg, np.float32(1e-30)).astype(np.float64))) / (r - 1.0)
    assert np.all(np.abs(w - wr) <= 8.0 * 2.0 ** -23 * (1.0 + expo) * wr + np.finfo(np.float32).tiny)
    assert np.array_equal(w == 0.0, wr == 0.0) and np.any(wr == 0.0) and np.any(wr > 0.0)
    _, n64 = ctrl.baseline_normalizer()
    assert abs(n64[0] - ref["normalizer"]) <= 1e-5 * ref["normalizer"]
    _parity.check_control(ctrl.getControlSeq().T, ref, K, T, 2)
    ctrl.close()


def test_exponential_path_and_final_clamp_of_control_one():
    """gamma = 0 keeps the exponential weights: the same costs and update as VanillaMPPI; after smoothing only
    control 1 is clamped (control 0 may leave [-1, 1] where the Savitzky-Golay taps overshoot)."""
    K, T = 2048, 48
    rng = np.random.default_rng(5)
    x0 = np.array([1.0, 4.0, 0.0, 0.0], np.float32)
    col = _controller(ColoredMPPIController, K, T)
    van = _controller(VanillaMPPIController, K, T)
    # large noise against tight ranges, so the smoothed sequence overshoots the clamp somewhere
    for c in (col, van):
        c.setSamplingParams(GaussianDistribution(std_dev=(3.0, 3.0)))
    state = rng.bit_generator.state
    ref = _solve(col, K, T, rng, x0)
    rng.bit_generator.state = state
    _solve(van, K, T, rng, x0)
    assert np.array_equal(col.sample_costs(), van.sample_costs())
    assert np.array_equal(col.sample_costs().view(np.uint32), ref["costs"].view(np.uint32))
    _parity.check_control(col.getControlSeq().T, ref, K, T, 2)
    u_col, u_van = col.getControlSeq(), van.getControlSeq()
    # the same smoothed sequence; Vanilla clamps both controls, ColoredMPPI control 1 only
    assert np.array_equal(u_col[1], u_van[1]) and np.all(np.abs(u_col[1]) <= 0.5)
    assert np.array_equal(np.clip(u_col[0], np.float32(-1.0), np.float32(1.0)), u_van[0])
    col.close()
    van.close()


def test_state_leash_holds_x0_near_the_nominal_state():
    K, T, jump = 1024, 40, 3
    ctrl = _controller(ColoredMPPIController, K, T)
    leash = np.array([0.05, 10.0, 0.0, 0.5], np.float32)
    for i, v in enumerate(leash):
        ctrl.setStateLeashLength(float(v), i)
    rng = np.random.default_rng(9)
    x0 = np.array([0.5, -1.0, 0.3, 0.1], np.float32)
    ctrl.computeControl(x0, 1)
    nominal = ctrl.getTargetStateSeq()[:, jump].copy()
    ctrl.slideControlSequence(jump)
    ctrl.setLeashActive(True)
    x1 = np.array([0.9, -1.5, 0.2, 0.0], np.float32)
    diff = np.abs(nominal - x1)
    expect = np.where(leash < diff, x1 + np.clip(nominal - x1, -leash, leash), nominal).astype(np.float32)
    ref = _solve(ctrl, K, T, rng, x1, x0_oracle=expect)  # the engine leashes x1; the oracle starts from the result
    assert np.array_equal(ctrl.sample_costs().view(np.uint32), ref["costs"].view(np.uint32))
    assert np.array_equal(ctrl.getTargetStateSeq()[:, 0], expect)
    ctrl.close()
