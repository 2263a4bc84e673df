"""RobustMPPIController over a caller's plugin pair (tests/plugins/di_plugins.cu) against the oracle's restatement of
the same pair (robust_mppi_controller.cu:480-744; rolloutRMPPIKernel and initEvalKernel, rmppi_kernels.cu:231-357,
666-861), given the same injected noise.  The reference's robust controller takes any Dynamics / Cost pair; here
both R-MPPI rollouts run the plugin's own step, its computeRunningCost with each system's own crash flag (a wall the
samples cross, cost.cuh:221-222) and, for di_constrained_quadratic, its own enforceConstraints with the state:
  * the first importance-sampler update takes the real state as the nominal state and solves the DDP gains around
    the nominal trajectory (di_quadratic: its computeGrad, within 1e-5 of the oracle's DDP);
  * a solve: the coupled rollout's costs and the written-back samples bit-identical to the oracle's; the sequences
    within 1e-5 of their term magnitude; the nominal state trajectory bit-identical;
  * a second update: candidates, strides, evaluation costs bit for bit, free energies, the chosen candidate and the
    slid nominal sequence.
TubeMPPIController over the same crash-wall pair (tube_mppi_controller.cu:158-296) against the oracle's Tube-MPPI
iteration: both distributions' costs bit for bit, baselines, the nominal-state decision and both sequences."""
import numpy as np
import pytest

import _parity
import _plugins
import oracle
from oracle import ddp as oddp
from mppi_generic_vendor_gb300 import DDPFeedback, DDPParams, GaussianDistribution
from mppi_generic_vendor_gb300.plugin import (PluginCost, PluginDynamics, PluginLibrary, PluginRobustMPPIController,
                                              PluginTubeMPPIController)
from test_gpu_rmppi import _line_weights
from test_gpu_tube import _check as _check_tube

pytestmark = pytest.mark.gpu

K, T, DT, N, J = 1024, 40, 0.02, 5, 32
SD = 0.8
Q = np.diag([4.0, 4.0, 1.0, 1.0]).astype(np.float32)
R = 0.5 * np.eye(2, dtype=np.float32)


def _cost(wall_x):
    c = _plugins.QuadraticWallCost()
    c.s_goal[:] = [1.5, -0.5, 0.0, 0.0]
    c.s_coeffs[:] = [1.0, 1.0, 0.1, 0.1]
    c.wall_x, c.crash_cost, c.terminal_coeff = wall_x, 50.0, 5.0
    return c


def _dyn_params(name):
    if name == "di_constrained_quadratic":
        return _plugins.DIConstrainedPlugin(0.1, 2.0, 0.5)
    return _plugins.DIPlugin(0.3)


@pytest.fixture(scope="module")
def plugin_path():
    return _plugins.library_path()


@pytest.mark.parametrize("threshold", [1e9, -1e9])
@pytest.mark.parametrize("name", ["di_quadratic", "di_constrained_quadratic"])
def test_plugin_rmppi_update_solve_update_matches_oracle(plugin_path, name, threshold):
    lib = PluginLibrary(plugin_path, name)
    dyn = PluginDynamics(lib, _dyn_params(name))
    dyn.setControlRanges([(-2.0, 2.0), (-2.0, 2.0)])
    cost = PluginCost(lib, _cost(0.45))
    fb = DDPFeedback(dyn, DT)
    fb.setParams(DDPParams(Q, None, R, 1))
    init = np.random.default_rng(2).uniform(-0.3, 0.3, (2, T)).astype(np.float32)
    sampler = GaussianDistribution(std_dev=(SD, SD), control_cost_coeff=(0.3, 0.3))
    ctrl = PluginRobustMPPIController(dyn, cost, fb, sampler, DT, 1, 1.0, 0.0, threshold, T, K,
                                      init_control_traj=init, num_candidate_nominal_states=N,
                                      num_eval_samples_per_candidate=J)
    mid = _plugins.ORACLE_MODEL[name]
    sd = np.full(2, SD, np.float32)
    rng = np.random.default_rng(7)
    eps = rng.standard_normal(K * T * 2).astype(np.float32)
    ctrl.injectNoise(np.concatenate([eps, rng.standard_normal(K * T * 2).astype(np.float32)]))
    dp, cp, sp, cc = ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.sampler_.to_c(), ctrl.constraints_
    x = np.array([0.1, -0.05, 0.9, 0.1], np.float32)
    # ---- 1. the first update
    ctrl.updateImportanceSamplingControl(x, 1)
    assert np.array_equal(ctrl.getNominalState(), x)
    fs = ctrl.getFeedbackState()
    gains = np.stack([fs.gain(t) for t in range(T)])
    assert np.all(np.isfinite(gains)) and np.any(gains != 0)
    if name == "di_quadratic":
        d = np.float32(0.3)

        def f(xs, us):
            xs, us = np.asarray(xs, np.float32), np.asarray(us, np.float32)
            return np.array([xs[2], xs[3], us[0] - d * xs[2], us[1] - d * xs[3]], np.float32)

        def df(xs, us):
            A_ = np.zeros((4, 4))
            A_[0, 2] = A_[1, 3] = 1.0
            A_[2, 2] = A_[3, 3] = -float(d)
            B_ = np.zeros((4, 2))
            B_[2, 0] = B_[3, 1] = 1.0
            return A_, B_

        lo, hi = np.array([-2.0, -2.0], np.float32), np.array([2.0, 2.0], np.float32)
        ref = oddp.ddp_gains(f, df, x, ctrl.getTargetStateSeq().T.copy(), ctrl.getNominalControlSeq().T.copy(), DT,
                             Q, np.eye(4, dtype=np.float32), R, 1, lo, hi)
        assert np.abs(gains - ref).max() <= 1e-5 * np.abs(ref).max()
    # ---- 2. the solve from a real state off the nominal one
    u_nom = ctrl.getNominalControlSeq().T.copy()
    x_nom = ctrl.getNominalState()
    x_real = (x + np.array([0.05, -0.03, 0.1, 0.05], np.float32)).astype(np.float32)
    ctrl.computeControl(x_real, 1)
    raw = oracle.gaussian_rewrite(eps, u_nom, sd, K, T, 2, 1)
    g_flat = gains.transpose(0, 2, 1).reshape(T, -1)
    cn, cr, un, ur = oracle.rmppi_rollout(mid, dp, cp, x_nom, x_real, raw, raw, u_nom, u_nom, g_flat, sp, cc, 1.0,
                                          0.0, threshold, K, T, DT)
    costs = ctrl.sample_costs().reshape(2, K)
    assert np.array_equal(costs[0].view(np.uint32), cn.view(np.uint32))
    assert np.array_equal(costs[1].view(np.uint32), cr.view(np.uint32))
    samples = ctrl.control_samples().reshape(2, K * T * 2)
    assert np.array_equal(samples[0], un) and np.array_equal(samples[1], ur)
    assert not np.array_equal(un, ur)
    # the wall at x = 0.45 is crossed: without it the oracle's costs change
    cn_free, cr_free, _, _ = oracle.rmppi_rollout(mid, dp, _cost(1e9), x_nom, x_real, raw, raw, u_nom, u_nom, g_flat,
                                                  sp, cc, 1.0, 0.0, threshold, K, T, DT)
    assert np.any(cr_free != cr) and np.any(cn_free != cn)
    if name == "di_constrained_quadratic":
        # the plugin's speed-dependent bound (below the handle's range of 2) binds on some written-back controls
        assert np.abs(ur).max() < 2.0 and np.abs(raw).max() > 2.0
    bn, _ = ctrl.baseline_normalizer()
    for i, (c, s, got) in enumerate([(cn, un, ctrl.getNominalControlSeq()), (cr, ur, ctrl.getControlSeq())]):
        w, b, n = oracle.weights(c, lambda_inv=np.float32(1.0))
        assert bn[i, 0] == b
        mean, _ = oracle.weighted_mean(w, np.float32(n), s, K, T, 2)
        ref = oracle.smooth(mean.astype(np.float32).reshape(T, 2))
        _parity.check_control(got.T, dict(control=ref, weights=w, normalizer=n, samples=s), K, T, 2)
    # the nominal state trajectory: each step's constraint (the plugin's own, with the state) and the plugin's step
    _, _, tr = oracle.rollout(mid, dp, cp, x_nom, ctrl.getNominalControlSeq().T.copy(), u_nom, sp, cc, 1.0, 0.0, 1,
                              T, DT, want_traj=True, state_dim=4)
    expect = np.concatenate([x_nom[None], tr.reshape(T, 4)[:-1].astype(np.float32)])
    assert np.array_equal(ctrl.getTargetStateSeq().T.view(np.uint32), expect.view(np.uint32))
    # ---- 3. the second update
    p = ctrl.getTargetStateSeq().T.copy()
    u_prev = ctrl.getNominalControlSeq().T.copy()
    x2 = np.array([0.16, -0.1, 0.95, 0.02], np.float32)
    ctrl.updateImportanceSamplingControl(x2, 1)
    best, stride, cand, strides, fe, evc = ctrl._candidates()
    w = _line_weights(N)
    exp_cand = (p[0][None, :] * w[0][:, None] + p[1][None, :] * w[1][:, None]) + x2[None, :] * w[2][:, None]
    assert np.array_equal(cand, exp_cand.astype(np.float32))
    raw_eval = oracle.gaussian_rewrite(eps, u_prev, sd, K, T, 2, 1)
    ref_eval = oracle.rmppi_eval(mid, dp, cp, cand, strides, J, raw_eval, u_prev, sp, cc, 1.0, 0.0, K, T, DT)
    assert np.array_equal(evc.view(np.uint32), ref_eval.view(np.uint32))
    base = ref_eval.min()
    with np.errstate(divide="ignore"):
        ref_fe = np.array([-1.0 * np.log(np.exp((base - ref_eval[i * J:(i + 1) * J]).astype(np.float32))
                                         .astype(np.float64).mean()) + base for i in range(N)])
    assert np.allclose(fe, ref_fe, rtol=1e-5, atol=1e-5)
    below = [i for i in range(N) if ref_fe[i] < threshold]
    exp_best = below[-1] if below else 0
    assert best == exp_best and stride == strides[exp_best]
    assert np.array_equal(ctrl.getNominalState(), cand[exp_best])
    slid = oracle.slide(u_prev, int(stride), np.zeros(2, np.float32), np.zeros(2, np.float32))
    assert np.array_equal(ctrl.getNominalControlSeq().T, slid)
    ctrl.close()


@pytest.mark.parametrize("threshold", [20.0, -1e9])
def test_plugin_tube_matches_oracle(plugin_path, threshold):
    lib = PluginLibrary(plugin_path, "di_quadratic")
    dyn = PluginDynamics(lib, _plugins.DIPlugin(0.3))
    dyn.setControlRanges([(-2.0, 2.0), (-2.0, 2.0)])
    ctrl = PluginTubeMPPIController(dyn, PluginCost(lib, _cost(0.45)), None, GaussianDistribution(std_dev=(SD, SD)),
                                    DT, 1, 1.0, 0.0, T, K, nominal_threshold=threshold)
    rng = np.random.default_rng(5)
    init = rng.uniform(-0.5, 0.5, (T, 2)).astype(np.float32)
    ctrl.setControlSeq(init.T)
    e = rng.standard_normal(K * T * 2).astype(np.float32)
    ctrl.injectNoise(np.concatenate([e, rng.standard_normal(K * T * 2).astype(np.float32)]))
    x = np.array([0.1, -0.05, 0.9, 0.1], np.float32)
    ctrl.computeControl(x, 1)
    ref = oracle.tube_compute_control(_plugins.ORACLE_MODEL["di_quadratic"], ctrl._dyn_arr[0], ctrl._cost_arr[0],
                                      ctrl.getParams(), ctrl.sampler_.to_c(), ctrl.constraints_, K, T, 2, 4, x, x,
                                      np.concatenate([e, e]), np.stack([init, init]))
    _check_tube(ctrl, ref, K, T)
    ctrl.close()
