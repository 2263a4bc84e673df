"""RobustMPPIController on the GPU against the oracle's restatement (robust_mppi_controller.cu:480-744;
rolloutRMPPIKernel and initEvalKernel, rmppi_kernels.cu:231-357, 666-861), given the same injected noise:
  * the first importance-sampler update takes the real state as the nominal state and computes the DDP gains around
    the nominal trajectory (bit for bit against the handle-free solver);
  * a solve: both distributions sample around the nominal sequence with one noise draw; the coupled rollout's costs
    (the nominal costs blending in the real system's) and the constrained samples (the real ones with the feedback)
    are bit-identical to the oracle's; the updated and smoothed sequences are within 1e-5 of their term magnitude;
  * a second update: candidate states and strides on the line search, the evaluation rollouts' costs bit for bit,
    the free energies, the chosen candidate (all below the threshold: the last; none: the previous choice), the nominal
    sequence slid by the chosen stride and the new gains.
Models: the double integrator with an obstacle, the cart-pole, the kinematic bicycle on a costmap (the costmap lookup
inside both R-MPPI kernels) and the 7-state dynamic bicycle on the same costmap."""
import numpy as np
import pytest

import _parity
import oracle
from _ddp import engine_gains
from mppi_generic_vendor_gb300 import (BicycleDynamics, BicycleSlipDynamics, CartpoleDynamics, CartpoleSwingupCost,
                                       CostmapCost, DDPFeedback, DDPParams, DoubleIntegratorDynamics,
                                       DoubleIntegratorObstacleCost, GaussianDistribution, RobustMPPIController)
from mppi_generic_vendor_gb300 import _abi as A
from mppi_generic_vendor_gb300.workloads import gaussian_bump_costmap

pytestmark = pytest.mark.gpu

K, T, DT, N, J = 1024, 40, 0.02, 5, 32
CMAP = gaussian_bump_costmap(3, size=128)  # 12.8 m square at 0.1 m cells


def _costmap_cost():
    return CostmapCost(map_coeff=1.0, speed_target=8.0, speed_coeff=1.0, steer_coeff=0.5, terminal_coeff=2.0,
                       costmap=CMAP, resolution=0.1, origin=(0.0, 0.0))


# (model id, dynamics, cost, control ranges, std dev, likelihood coefficient, x, disturbance, second state)
MODELS = {
    "double_integrator": (A.MODEL_DOUBLE_INTEGRATOR, DoubleIntegratorDynamics,
                          lambda: DoubleIntegratorObstacleCost(goal=(1.5, -0.5, 0.0, 0.0), coeff=(1.0, 1.0, 0.1, 0.1),
                                                               terminal_coeff=5.0, obstacles=[(0.7, 0.0, 0.3)],
                                                               obstacle_cost=100.0),
                          [(-2.0, 2.0)] * 2, 0.6, 0.3, [0.1, -0.05, 0.3, 0.1], [0.05, -0.03, 0.1, 0.05],
                          [0.16, -0.1, 0.35, 0.02]),
    "cartpole": (A.MODEL_CARTPOLE, CartpoleDynamics, lambda: CartpoleSwingupCost(), [(-5.0, 5.0)], 1.0, 0.2,
                 [0.0, 0.1, 2.6, -0.2], [0.02, -0.05, 0.08, 0.1], [0.05, 0.0, 2.7, 0.3]),
    "bicycle_costmap": (A.MODEL_BICYCLE_COSTMAP, lambda: BicycleDynamics(2.5), _costmap_cost, [(-3.0, 3.0), (-1.0, 1.0)],
                        0.5, 0.2, [6.0, 5.0, 0.4, 4.0], [0.1, -0.08, 0.05, 0.3], [6.3, 5.2, 0.38, 4.4]),
    "bicycle_slip": (A.MODEL_BICYCLE_SLIP, BicycleSlipDynamics, _costmap_cost, [(-3.0, 3.0), (-0.5, 0.5)], 0.4, 0.2,
                     [6.0, 5.0, 0.2, 6.0, 0.0, 0.0, 0.0], [0.1, -0.05, 0.02, 0.2, 0.05, 0.01, 0.0],
                     [6.3, 5.1, 0.22, 6.2, 0.02, 0.01, 0.0]),
}


def _Q(S):
    return np.diag([4.0, 4.0, 1.0, 1.0] + [1.0] * (S - 4)).astype(np.float32)


def _map(name):
    return (CMAP, 0.1, (0.0, 0.0)) if name.startswith("bicycle") else None


def _controller(name, threshold):
    mid, dyn_cls, cost_fn, ranges, sd, coeff = MODELS[name][:6]
    dyn = dyn_cls()
    Cd = dyn.CONTROL_DIM
    dyn.setControlRanges(ranges)
    fb = DDPFeedback(dyn, DT)
    fb.setParams(DDPParams(_Q(dyn.STATE_DIM), None, 0.5 * np.eye(Cd, dtype=np.float32), 1))
    sampler = GaussianDistribution(std_dev=(sd,) * Cd, control_cost_coeff=(coeff,) * Cd)
    init = np.random.default_rng(2).uniform(-0.3, 0.3, (Cd, T)).astype(np.float32)
    return RobustMPPIController(dyn, cost_fn(), fb, sampler, DT, 1, 1.0, 0.0, threshold, T, K, init_control_traj=init,
                                num_candidate_nominal_states=N, num_eval_samples_per_candidate=J)


def _gains(ctrl):
    fs = ctrl.getFeedbackState()
    return np.stack([fs.gain(t) for t in range(T)])


def _check_gains(ctrl, x):
    Cd = ctrl.Cdim
    lo, hi = np.array(ctrl.constraints_.lower[:Cd], np.float32), np.array(ctrl.constraints_.upper[:Cd], np.float32)
    S = ctrl.S
    st, host = engine_gains(ctrl.model_id, ctrl._dyn_arr[0], x, ctrl.getTargetStateSeq().T.copy(),
                            ctrl.getNominalControlSeq().T.copy(), DT, _Q(S), np.eye(S, dtype=np.float32),
                            0.5 * np.eye(Cd, dtype=np.float32), 1, lo, hi)
    assert st == A.MPPI_OK
    got = _gains(ctrl)
    assert np.array_equal(got.view(np.uint32), host.view(np.uint32))
    assert np.any(got != 0)
    return got


def _line_weights(n):
    h = n // 2
    w = np.zeros((3, n), np.float32)
    for i in range(h + 1):
        w[0, i] = np.float32(1) - np.float32(i) / np.float32(h)
        w[1, i] = np.float32(i) / np.float32(h)
    for i in range(1, h + 1):
        w[1, h + i] = np.float32(1) - np.float32(i) / np.float32(h)
        w[2, h + i] = np.float32(i) / np.float32(h)
    return w


@pytest.mark.parametrize("threshold", [1e9, -1e9])
@pytest.mark.parametrize("name", list(MODELS))
def test_rmppi_update_solve_update_matches_oracle(name, threshold):
    ctrl = _controller(name, threshold)
    mid, Cd = ctrl.model_id, ctrl.Cdim
    sd = np.full(Cd, MODELS[name][4], np.float32)
    rng = np.random.default_rng(7)
    eps = rng.standard_normal(K * T * Cd).astype(np.float32)
    # one noise draw serves both distributions (use_same_noise_for_all_distributions): the second half is ignored
    ctrl.injectNoise(np.concatenate([eps, rng.standard_normal(K * T * Cd).astype(np.float32)]))
    x = np.array(MODELS[name][6], np.float32)
    dyn, cost, sp, cc = ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.sampler_.to_c(), ctrl.constraints_
    # ---- 1. the first update: the nominal state is the real state; gains around the nominal trajectory
    ctrl.updateImportanceSamplingControl(x, 1)
    assert np.array_equal(ctrl.getNominalState(), x)
    gains = _check_gains(ctrl, x)
    # ---- 2. the solve
    u_nom = ctrl.getNominalControlSeq().T.copy()
    x_nom = ctrl.getNominalState()
    x_real = (x + np.array(MODELS[name][7], np.float32)).astype(np.float32)  # disturbed off the nominal
    ctrl.computeControl(x_real, 1)
    raw = oracle.gaussian_rewrite(eps, u_nom, sd, K, T, Cd, 1)
    cn, cr, un, ur = oracle.rmppi_rollout(mid, dyn, cost, x_nom, x_real, raw, raw, u_nom, u_nom,
                                          gains.transpose(0, 2, 1).reshape(T, -1), sp, cc, 1.0, 0.0, threshold, K,
                                          T, DT, costmap=_map(name))
    costs = ctrl.sample_costs().reshape(2, K)
    assert np.array_equal(costs[0].view(np.uint32), cn.view(np.uint32))
    assert np.array_equal(costs[1].view(np.uint32), cr.view(np.uint32))
    samples = ctrl.control_samples().reshape(2, K * T * Cd)
    assert np.array_equal(samples[0], un) and np.array_equal(samples[1], ur)
    assert not np.array_equal(un, ur)  # the feedback moved the real system's controls
    bn, _ = ctrl.baseline_normalizer()
    for d, (c, s, got) in enumerate([(cn, un, ctrl.getNominalControlSeq()), (cr, ur, ctrl.getControlSeq())]):
        w, b, n = oracle.weights(c, lambda_inv=np.float32(1.0))
        assert bn[d, 0] == b
        mean, _ = oracle.weighted_mean(w, np.float32(n), s, K, T, Cd)
        ref = oracle.smooth(mean.astype(np.float32).reshape(T, Cd))
        _parity.check_control(got.T, dict(control=ref, weights=w, normalizer=n, samples=s), K, T, Cd)
    # the nominal state trajectory: from the nominal state along the (constrained) nominal sequence
    traj = [x_nom]
    for t in range(T - 1):
        u_c = oracle.enforce_constraints(ctrl.getNominalControlSeq().T[t], Cd, cc)
        traj.append(oracle.step_state(mid, dyn, cost, traj[-1], u_c, DT))
    assert np.array_equal(ctrl.getTargetStateSeq().T, np.stack(traj))
    # ---- 3. the second update from a disturbed real state
    p = ctrl.getTargetStateSeq().T.copy()
    u_prev = ctrl.getNominalControlSeq().T.copy()
    x2 = np.array(MODELS[name][8], np.float32)
    S = ctrl.S
    ctrl.updateImportanceSamplingControl(x2, 1)
    best, stride, cand, strides, fe, evc = ctrl._candidates()
    w = _line_weights(N)
    exp_cand = ((p[0][None, :] * w[0][:, None] + p[1][None, :] * w[1][:, None]) + x2[None, :] * w[2][:, None])
    assert np.array_equal(cand, exp_cand.astype(np.float32))
    # Eigen's round (std::round) takes halves away from zero
    exp_strides = np.floor(((np.float32(0) * w[0] + np.float32(1) * w[1]) + np.float32(1) * w[2]) + 0.5).astype(np.int32)
    assert np.array_equal(strides, exp_strides)
    raw_eval = oracle.gaussian_rewrite(eps, u_prev, sd, K, T, Cd, 1)
    ref_eval = oracle.rmppi_eval(mid, dyn, cost, cand, strides, J, raw_eval, u_prev, sp, cc, 1.0, 0.0, K, T, DT,
                                 costmap=_map(name))
    assert np.array_equal(evc.view(np.uint32), ref_eval.view(np.uint32))
    # computeBestIndex: exponentials in FP32 (a candidate whose samples all lie far above the best one sums to zero
    # and gets an infinite free energy), the last candidate below the threshold, else the previous choice (0)
    base = ref_eval.min()
    with np.errstate(divide="ignore"):
        ref_fe = np.array([-1.0 * np.log(np.exp((base - ref_eval[i * J:(i + 1) * J]).astype(np.float32))
                                         .astype(np.float64).mean()) + base for i in range(N)])
    assert np.allclose(fe, ref_fe, rtol=1e-5, atol=1e-5)
    below = [i for i in range(N) if ref_fe[i] < threshold]
    exp_best = below[-1] if below else 0
    assert (exp_best == N - 1) if threshold > 0 else (exp_best == 0)
    assert best == exp_best and stride == strides[exp_best]
    nom = np.zeros(1, np.int32)
    A.call("mppi_get_nominal_state_used", ctrl._h, nom.ctypes.data_as(A._IP))
    assert nom[0] == exp_best
    assert np.array_equal(ctrl.getNominalState(), cand[exp_best])
    slid = oracle.slide(u_prev, int(stride), np.zeros(Cd, np.float32), np.zeros(Cd, np.float32))
    assert np.array_equal(ctrl.getNominalControlSeq().T, slid)
    _check_gains(ctrl, x2)
    # slideControlSequence and computeFeedback do nothing on a robust controller
    before = ctrl.getControlSeqs()
    ctrl.slideControlSequence(3)
    ctrl.computeFeedback(x)
    after = ctrl.getControlSeqs()
    assert all(np.array_equal(a, b) for a, b in zip(before, after))
    ctrl.close()


def test_rmppi_rejects_bad_candidate_counts():
    from mppi_generic_vendor_gb300 import MPPIError

    dyn = DoubleIntegratorDynamics()
    with pytest.raises(MPPIError):
        RobustMPPIController(dyn, DoubleIntegratorObstacleCost(), None, GaussianDistribution(std_dev=(0.5, 0.5)), DT,
                             1, 1.0, 0.0, 1000.0, T, K, num_candidate_nominal_states=4)
    with pytest.raises(MPPIError):
        RobustMPPIController(dyn, DoubleIntegratorObstacleCost(), None, GaussianDistribution(std_dev=(0.5, 0.5)), DT,
                             1, 1.0, 0.0, 1000.0, T, 256, num_candidate_nominal_states=9,
                             num_eval_samples_per_candidate=64)
