"""Plugin pairs defined outside the engine's sources (tests/plugins/di_plugins.cu, written against
include/mppi_gb_plugin.cuh) run through the ordinary C entry points and match the oracle's restatement of the same
pair bit for bit: per-sample costs, the baseline, the constrained samples, the nominal state trajectory (the
plugin's own step on the host twin) and, from the sampled-trajectory read-out, every step's output, running cost and
crash flag (the crash argument of computeRunningCost, cost.cuh:221-222)."""
import ctypes as C

import numpy as np
import pytest

import _parity
import _plugins
import oracle
from mppi_generic_vendor_gb300 import GaussianDistribution, MPPIError
from mppi_generic_vendor_gb300 import _abi as A
from mppi_generic_vendor_gb300.plugin import PluginCost, PluginDynamics, PluginLibrary, PluginMPPIController

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plugin_path():
    return _plugins.library_path()


def _cost(goal, wall=1.5, crash_cost=50.0, terminal=5.0):
    c = _plugins.QuadraticWallCost()
    c.s_goal[:] = [float(v) for v in goal]
    c.s_coeffs[:] = [1.0, 1.0, 0.1, 0.1]
    c.wall_x, c.crash_cost, c.terminal_coeff = wall, crash_cost, terminal
    return c


def _controller(path, name, damping, goals, Ks, Ts, lam=1.0, ranges=((-2.0, 2.0), (-2.0, 2.0))):
    lib = PluginLibrary(path, name)
    dyn = PluginDynamics(lib, _plugins.DIPlugin(damping))
    dyn.setControlRanges(list(ranges))
    costs = [PluginCost(lib, _cost(g)) for g in goals]
    return PluginMPPIController(dyn, costs, GaussianDistribution(std_dev=(0.8, 0.8)), Ks, Ts, dt=0.05, max_iter=1,
                                lambda_=lam)


@pytest.mark.parametrize("name,damping", [("di_quadratic", 0.0), ("di_quadratic", 0.4),
                                          ("di_symplectic_quadratic", 0.25)])
def test_plugin_controller_matches_oracle(plugin_path, name, damping):
    rng = np.random.default_rng(7)
    Ks, Ts = [2048, 1000, 512], [64, 40, 32]
    goals = [(2.0, 0.5, 0.0, 0.0), (1.0, -1.0, 0.0, 0.0), (0.0, 1.0, 0.0, 0.0)]
    ctrl = _controller(plugin_path, name, damping, goals, Ks, Ts)
    model, S, Cd, O = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    A.call("mppi_get_model_dims", ctrl._h, C.byref(model), C.byref(S), C.byref(Cd), C.byref(O))
    assert (model.value, S.value, Cd.value, O.value) == (A.MODEL_PLUGIN, 4, 2, 4)
    eps = [rng.standard_normal(K * T * 2).astype(np.float32) for K, T in zip(Ks, Ts)]
    init = [rng.uniform(-0.5, 0.5, (T, 2)).astype(np.float32) for T in Ts]
    x0 = [np.array([0.0, 0.0, 0.5, 0.2], np.float32), np.array([0.5, 0.5, 0.0, 0.0], np.float32),
          np.array([1.2, 0.0, 0.8, 0.0], np.float32)]
    ctrl.setControlSeqs([u.T for u in init])
    ctrl.injectNoise(np.concatenate(eps))
    ctrl.computeControl(np.concatenate(x0), 1)
    costs, samples, ctl = ctrl.sample_costs(), ctrl.control_samples(), ctrl.getControlSeqs()
    states = ctrl.getTargetStateSeqs()
    bn, _ = ctrl.baseline_normalizer()
    koff, uoff = np.concatenate([[0], np.cumsum(Ks)]), np.concatenate([[0], np.cumsum(np.array(Ks) * Ts * 2)])
    crashed = 0
    for i, (K, T) in enumerate(zip(Ks, Ts)):
        ref = oracle.compute_control(_plugins.ORACLE_MODEL[name], ctrl._dyn_arr[i], ctrl._cost_arr[i],
                                     ctrl.getParams(), ctrl.sampler_.to_c(), ctrl.constraints_, K, T, 2, 4, x0[i],
                                     eps[i], init[i])
        assert np.array_equal(costs[koff[i]:koff[i + 1]].view(np.uint32), ref["costs"].view(np.uint32)), i
        assert np.array_equal(samples[uoff[i]:uoff[i + 1]].view(np.uint32), ref["samples"].view(np.uint32)), i
        assert bn[i, 0] == ref["baseline"]
        _parity.check_control(ctl[i].T, ref, K, T, 2)
        # the nominal state trajectory: the plugin's own step on the host, along the engine's updated sequence
        _, _, tr = oracle.rollout(_plugins.ORACLE_MODEL[name], ctrl._dyn_arr[i], ctrl._cost_arr[i], x0[i],
                                  np.ascontiguousarray(ctl[i].T), init[i], ctrl.sampler_.to_c(), ctrl.constraints_,
                                  1.0, 0.0, 1, T, 0.05, want_traj=True, state_dim=4)
        expect = np.concatenate([x0[i][None], tr.reshape(T, 4)[:-1].astype(np.float32)])
        assert np.array_equal(states[i].T.view(np.uint32), expect.view(np.uint32)), i
        # the crash wall is reached by part of the samples
        _, _, traj = oracle.rollout(_plugins.ORACLE_MODEL[name], ctrl._dyn_arr[i], ctrl._cost_arr[i], x0[i],
                                    ref["samples"], init[i], ctrl.sampler_.to_c(), ctrl.constraints_, 1.0, 0.0, K, T,
                                    0.05, want_traj=True, state_dim=4)
        crashed += int(np.any(traj.reshape(K, T, 4)[:, :, 0] > 1.5, axis=1).sum())
    assert crashed > 0
    ctrl.close()


def test_plugin_sampled_trajectories_report_outputs_costs_and_crash(plugin_path):
    K, T = 1024, 48
    rng = np.random.default_rng(3)
    ctrl = _controller(plugin_path, "di_quadratic", 0.1, [(2.0, 0.0, 0.0, 0.0)], [K], [T])
    eps = rng.standard_normal(K * T * 2).astype(np.float32)
    x0 = np.array([0.8, 0.0, 1.0, 0.0], np.float32)
    ctrl.injectNoise(eps)
    ctrl.computeControl(x0, 1)
    ctrl.setPercentageSampledControlTrajectories(0.05)
    ctrl.setTopNSampledControlTrajectories(8)
    ctrl.calculateSampledStateTrajectories(0, seed=2)
    idx = ctrl.sampled_indices_
    samples = ctrl.control_samples().reshape(K, T, 2)
    chosen = np.ascontiguousarray(samples[idx])
    mean0 = np.zeros((T, 2), np.float32)
    r32, _, traj = oracle.rollout(_plugins.ORACLE_MODEL["di_quadratic"], ctrl._dyn_arr[0], ctrl._cost_arr[0], x0,
                                  chosen, mean0, ctrl.sampler_.to_c(), ctrl.constraints_, 1.0, 0.0, len(idx), T, 0.05,
                                  want_traj=True, state_dim=4)
    traj = traj.reshape(len(idx), T, 4).astype(np.float32)
    got = np.stack([s.T for s in ctrl.getSampledOutputTrajectories()])
    assert np.array_equal(got.view(np.uint32), traj.view(np.uint32))
    crash = np.stack(ctrl.getSampledCrashStatus())
    expect = np.maximum.accumulate(traj[:, :, 0] > 1.5, axis=1).astype(np.int32)
    assert np.array_equal(crash, expect) and crash.any() and not crash.all()
    # the step costs and terminal cost rebuild each sample's cost in the rollout's order
    steps = np.stack(ctrl.getSampledCostTrajectories())
    for j, k in enumerate(idx):
        running = np.float32(0.0)
        for t in range(T):
            running = np.float32(running + steps[j, t])
        total = np.float32(running / np.float32(T)) + np.float32(ctrl.sampled_terminal_costs_[j] / np.float32(T))
        assert np.float32(total) == ctrl.sample_costs()[k]
    ctrl.close()


def test_plugin_rejects_wrong_parameter_blocks(plugin_path):
    lib = PluginLibrary(plugin_path, "di_quadratic")
    with pytest.raises(ValueError):
        PluginCost(lib, _plugins.DIPlugin())
    dyn = PluginDynamics(lib, _plugins.DIPlugin(0.0))
    ctrl = PluginMPPIController(dyn, PluginCost(lib, _cost((1, 1, 0, 0))), GaussianDistribution(std_dev=(1.0, 1.0)),
                                [256], [16])
    with pytest.raises(MPPIError):
        ctrl.setRolloutMode(4)  # the plugin rollout is the sampler kernel followed by the plugin kernel
    ctrl.close()


def test_plugin_own_enforce_constraints_match_oracle(plugin_path):
    """A plugin that defines enforceConstraints(state, control): the samples leave the sampler unconstrained, each
    rollout step constrains its control with the current state and writes it back (rolloutKernel,
    mppi_common.cu:114-123); the final pass constrains the smoothed sequence with a zero state (mppi_controller.cu:
    222-226) and the nominal state trajectory constrains the smoothed sequence with the state
    (controller.cuh:676-680).  Costs, written-back samples, baseline and the state trajectory bit-identical to the
    oracle's restatement of the same pair; the update within 1e-5 of its term magnitude."""
    name = "di_constrained_quadratic"
    rng = np.random.default_rng(11)
    Ks, Ts = [2048, 700], [48, 30]
    lib = PluginLibrary(plugin_path, name)
    dpar = _plugins.DIConstrainedPlugin(0.1, 2.0, 0.5)
    dyn = PluginDynamics(lib, dpar)
    dyn.setControlRanges([(-2.0, 2.0), (-2.0, 2.0)])  # the handle's ranges: replaced by the plugin's method
    goals = [(2.0, 0.5, 0.0, 0.0), (-1.0, 1.0, 0.0, 0.0)]
    costs = [PluginCost(lib, _cost(g, wall=3.0)) for g in goals]
    ctrl = PluginMPPIController(dyn, costs, GaussianDistribution(std_dev=(1.2, 1.2)), Ks, Ts, dt=0.05, max_iter=1,
                                lambda_=1.0)
    eps = [rng.standard_normal(K * T * 2).astype(np.float32) for K, T in zip(Ks, Ts)]
    init = [rng.uniform(-0.5, 0.5, (T, 2)).astype(np.float32) for T in Ts]
    x0 = [np.array([0.0, 0.0, 1.5, -0.5], np.float32), np.array([0.5, 0.5, -2.5, 0.0], np.float32)]
    ctrl.setControlSeqs([u.T for u in init])
    ctrl.injectNoise(np.concatenate(eps))
    ctrl.computeControl(np.concatenate(x0), 1)
    got_costs, samples, ctl = ctrl.sample_costs(), ctrl.control_samples(), ctrl.getControlSeqs()
    states = ctrl.getTargetStateSeqs()
    bn, _ = ctrl.baseline_normalizer()
    koff, uoff = np.concatenate([[0], np.cumsum(Ks)]), np.concatenate([[0], np.cumsum(np.array(Ks) * Ts * 2)])
    bound_active = 0
    for i, (K, T) in enumerate(zip(Ks, Ts)):
        ref = oracle.compute_control(_plugins.ORACLE_MODEL[name], ctrl._dyn_arr[i], ctrl._cost_arr[i],
                                     ctrl.getParams(), ctrl.sampler_.to_c(), ctrl.constraints_, K, T, 2, 4, x0[i],
                                     eps[i], init[i])
        assert np.array_equal(got_costs[koff[i]:koff[i + 1]].view(np.uint32), ref["costs"].view(np.uint32)), i
        s = samples[uoff[i]:uoff[i + 1]]
        assert np.array_equal(s.view(np.uint32), ref["samples"].view(np.uint32)), i
        assert bn[i, 0] == ref["baseline"]
        _parity.check_control(ctl[i].T, ref, K, T, 2)
        # the nominal state trajectory: the plugin's constraint with the state, then its step, along the engine's
        # smoothed sequence (the final zero-state pass, a clamp to 2, leaves it unchanged here)
        assert np.all(np.abs(ctl[i]) < 2.0)
        _, _, tr = oracle.rollout(_plugins.ORACLE_MODEL[name], ctrl._dyn_arr[i], ctrl._cost_arr[i], x0[i],
                                  np.ascontiguousarray(ctl[i].T), init[i], ctrl.sampler_.to_c(), ctrl.constraints_,
                                  1.0, 0.0, 1, T, 0.05, want_traj=True, state_dim=4)
        expect = np.concatenate([x0[i][None], tr.reshape(T, 4)[:-1].astype(np.float32)])
        assert np.array_equal(states[i].T.view(np.uint32), expect.view(np.uint32)), i
        assert np.allclose(states[i].T, ref["state_seq"], rtol=1e-4, atol=1e-5)
        # the speed-dependent bound binds below the handle's range of 2: recompute it from each step's state
        _, _, traj = oracle.rollout(_plugins.ORACLE_MODEL[name], ctrl._dyn_arr[i], ctrl._cost_arr[i], x0[i], s.copy(),
                                    init[i], ctrl.sampler_.to_c(), ctrl.constraints_, 1.0, 0.0, K, T, 0.05,
                                    want_traj=True, state_dim=4)
        traj = traj.reshape(K, T, 4).astype(np.float32)
        before = np.concatenate([np.broadcast_to(x0[i], (K, 1, 4)), traj[:, :-1]], axis=1)
        amax = np.maximum(np.float32(0.5), np.float32(2.0) - np.float32(0.5) * np.abs(before[:, :, 2:4]))
        a = np.abs(s.reshape(K, T, 2))
        assert np.all(a <= amax)
        bound_active += int(np.sum((a == amax) & (amax < 2.0)))
        # the final pass with a zero state: every control within max(0.5, a_max) = 2
        assert np.all(np.abs(ctl[i]) <= 2.0)
    assert bound_active > 0
    ctrl.close()
