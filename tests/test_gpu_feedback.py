"""The DDP feedback controller behind a handle (Controller::initFeedback / computeFeedback / getFeedbackControl /
computeFeedbackPropagatedStateSeq, controller.cuh:265-269,495-571; DDPFeedback, ddp.cu:48-120) on trajectories solved
on the GPU: the gains equal the handle-free host solver's on the same nominal trajectory bit for bit and the oracle's
restatement within 1e-5 of their scale, the feedback control is K_t (x - goal) in FP32, the feedback-propagated
states equal the oracle's model steps bit for bit, Tube-MPPI tracks its nominal system, and a plugin's computeGrad
and the forward-difference fallback both reach the oracle."""
import ctypes as C

import numpy as np
import pytest

import _plugins
import oracle
from _ddp import engine_gains, feedback_control
from oracle import ddp as oddp
from mppi_generic_vendor_gb300 import (CartpoleDynamics, CartpoleSwingupCost, DDPFeedback, DDPParams,
                                       DoubleIntegratorDynamics, DoubleIntegratorObstacleCost, GaussianDistribution,
                                       TubeMPPIController, VanillaMPPIController)
from mppi_generic_vendor_gb300 import _abi as A
from mppi_generic_vendor_gb300.plugin import PluginCost, PluginDynamics, PluginLibrary, PluginMPPIController

pytestmark = pytest.mark.gpu


def _gains_array(state, T, Cd, S):
    return np.stack([state.gain(t) for t in range(T)])


def _propagated(model, dyn, cost, x_first, xt, un, K, dt):
    """Controller::computeFeedbackPropagatedStateSeq through the oracle's model steps (no constraints)."""
    T, S = xt.shape
    out = np.zeros((T, S), np.float32)
    x = np.asarray(x_first, np.float32).copy()
    out[0] = x
    for t in range(T - 1):
        u = (un[t] + feedback_control(K[t], x, xt[t])).astype(np.float32)
        x = oracle.step_state(model, dyn, cost, x, u, dt)
        out[t + 1] = x
    return out


def test_vanilla_cartpole_feedback():
    K, T, dt = 1024, 60, 0.02
    dyn = CartpoleDynamics()
    dyn.setControlRanges([(-5.0, 5.0)])
    cost = CartpoleSwingupCost()
    fb = DDPFeedback(dyn, dt)
    Q = np.diag([10.0, 1.0, 50.0, 1.0]).astype(np.float32)
    Qf = np.diag([20.0, 2.0, 100.0, 2.0]).astype(np.float32)
    R = np.diag([0.1]).astype(np.float32)
    fb.setParams(DDPParams(Q, Qf, R, 1))
    ctrl = VanillaMPPIController(dyn, cost, fb, GaussianDistribution(std_dev=(1.0,)), dt, 1, 1.0, 0.0, T, K)
    x0 = np.array([0.0, 0.0, 2.6, 0.0], np.float32)
    for _ in range(3):
        ctrl.computeControl(x0, 1)
    # off by default for a vanilla controller: computeFeedback leaves the gains at zero
    assert not ctrl.getFeedbackEnabled()
    ctrl.computeFeedback(x0)
    assert not np.any(ctrl.getFeedbackState().fb_gain_traj_)
    assert not np.any(ctrl.getFeedbackControl(x0 + 1.0, x0, 3))
    ctrl.initFeedback()
    assert ctrl.getFeedbackEnabled()
    on = C.c_int()
    A.call("mppi_get_feedback_enabled", ctrl._h, C.byref(on))
    assert on.value == 1
    x_start = (x0 + np.array([0.02, -0.05, -0.04, 0.1], np.float32)).astype(np.float32)
    ctrl.computeFeedback(x_start)
    got = _gains_array(ctrl.getFeedbackState(), T, 1, 4)
    xt, un = ctrl.getTargetStateSeq().T.copy(), ctrl.getControlSeq().T.copy()
    lo, hi = np.array([-5.0], np.float32), np.array([5.0], np.float32)
    st, host = engine_gains(A.MODEL_CARTPOLE, ctrl._dyn_arr[0], x_start, xt, un, dt, Q, Qf, R, 1, lo, hi)
    assert st == A.MPPI_OK
    assert np.array_equal(got.view(np.uint32), host.view(np.uint32))
    f, df = oddp.model_functions(A.MODEL_CARTPOLE, ctrl._dyn_arr[0], ctrl._cost_arr[0])
    ref = oddp.ddp_gains(f, df, x_start, xt, un, dt, Q, Qf, R, 1, lo, hi)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    # the feedback control, and its blend between steps as the plant applies it
    x = (xt[7] + np.array([0.01, 0.02, -0.03, 0.05], np.float32)).astype(np.float32)
    u = ctrl.getFeedbackControl(x, xt[7], 7)
    assert np.array_equal(u, feedback_control(got[7], x, xt[7]))
    fs = ctrl.getFeedbackState()
    mid = ctrl.interpolateFeedback(x, xt[7], 7.5 * dt, fs)
    assert np.allclose(mid, 0.5 * (got[7] @ (x - xt[7])) + 0.5 * (got[8] @ (x - xt[7])), rtol=1e-5, atol=1e-6)
    cur = ctrl.getCurrentControl(x, 7.5 * dt, xt[7], un.T, fs)
    assert np.allclose(cur, np.clip(0.5 * un[7] + 0.5 * un[8] + mid, -5.0, 5.0), rtol=1e-5, atol=1e-6)
    # the state trajectory under nominal control plus feedback, from the state the solve started at
    ctrl.computeFeedbackPropagatedStateSeq()
    prop = ctrl.getFeedbackPropagatedStateSeq().T
    expected = _propagated(A.MODEL_CARTPOLE, ctrl._dyn_arr[0], ctrl._cost_arr[0], xt[0], xt, un, got, dt)
    assert np.array_equal(prop.view(np.uint32), expected.view(np.uint32))
    # disabling keeps the last gains; enabling again resets them (initTrackingController)
    ctrl.disableFeedbackController()
    assert not ctrl.getFeedbackEnabled()
    assert np.array_equal(_gains_array(ctrl.getFeedbackState(), T, 1, 4), got)
    ctrl.initFeedback()
    assert not np.any(ctrl.getFeedbackState().fb_gain_traj_)
    ctrl.close()


def test_tube_feedback_tracks_the_nominal_system():
    K, T, dt = 1024, 40, 0.02
    dyn = DoubleIntegratorDynamics()
    dyn.setControlRanges([(-2.0, 2.0), (-2.0, 2.0)])
    cost = DoubleIntegratorObstacleCost(goal=(1.5, -0.5, 0.0, 0.0), coeff=(1.0, 1.0, 0.1, 0.1), terminal_coeff=5.0)
    fb = DDPFeedback(dyn, dt)
    Q = np.diag([5.0, 5.0, 1.0, 1.0]).astype(np.float32)
    R = np.diag([0.2, 0.2]).astype(np.float32)
    fb.setParams(DDPParams(Q, None, R, 1))
    # a threshold no baseline beats: the nominal system is always kept, so it differs from the actual one
    ctrl = TubeMPPIController(dyn, cost, fb, GaussianDistribution(std_dev=(0.6, 0.6)), dt, 1, 1.0, 0.0, T, K,
                              nominal_threshold=-1e9)
    assert ctrl.getFeedbackEnabled()  # Tube-MPPI turns it on at construction
    ctrl.computeControl(np.zeros(4, np.float32), 1)
    ctrl.slideControlSequence(1)
    x_actual = np.array([0.08, -0.05, 0.3, -0.2], np.float32)
    ctrl.computeControl(x_actual, 1)
    assert ctrl.nominalStateUsed() == 1
    nom_x, nom_u = ctrl.getTargetStateSeq().T.copy(), ctrl.getControlSeq().T.copy()
    assert not np.array_equal(nom_x[0], x_actual)
    ctrl.computeFeedback(x_actual)
    got = _gains_array(ctrl.getFeedbackState(), T, 2, 4)
    lo, hi = np.array([-2.0, -2.0], np.float32), np.array([2.0, 2.0], np.float32)
    st, host = engine_gains(A.MODEL_DOUBLE_INTEGRATOR, ctrl._dyn_arr[0], x_actual, nom_x, nom_u, dt, Q,
                            np.eye(4, dtype=np.float32), R, 1, lo, hi)
    assert st == A.MPPI_OK
    assert np.array_equal(got.view(np.uint32), host.view(np.uint32))
    ctrl.computeFeedbackPropagatedStateSeq()
    prop = ctrl.getFeedbackPropagatedStateSeq().T
    expected = _propagated(A.MODEL_DOUBLE_INTEGRATOR, ctrl._dyn_arr[0], ctrl._cost_arr[0],
                           ctrl.getActualStateSeq()[:, 0], nom_x, nom_u, got, dt)
    assert np.array_equal(prop.view(np.uint32), expected.view(np.uint32))
    ctrl.close()


@pytest.mark.parametrize("name", ["di_quadratic", "di_symplectic_quadratic"])
def test_plugin_feedback_jacobians(name):
    """di_quadratic defines computeGrad; di_symplectic_quadratic does not, so the controller differentiates the
    step's derivative forward (ModelWrapperDDP::df); both solve the oracle's problem."""
    path = _plugins.library_path()
    lib = PluginLibrary(path, name)
    damping = 0.3
    dyn = PluginDynamics(lib, _plugins.DIPlugin(damping))
    dyn.setControlRanges([(-2.0, 2.0), (-2.0, 2.0)])
    c = _plugins.QuadraticWallCost()
    c.s_goal[:] = [1.0, 0.5, 0.0, 0.0]
    c.s_coeffs[:] = [1.0, 1.0, 0.1, 0.1]
    c.wall_x, c.crash_cost, c.terminal_coeff = 5.0, 50.0, 5.0
    K, T, dt = 1024, 32, 0.05
    ctrl = PluginMPPIController(dyn, [PluginCost(lib, c)], GaussianDistribution(std_dev=(0.8, 0.8)), [K], [T], dt=dt,
                                max_iter=1, lambda_=1.0)
    Q = np.diag([3.0, 3.0, 0.5, 0.5]).astype(np.float32)
    R = np.diag([0.1, 0.1]).astype(np.float32)
    ctrl.setFeedbackParams(DDPParams(Q, Q, R, 1))
    ctrl.initFeedback()
    x0 = np.array([0.0, 0.0, 0.2, 0.0], np.float32)
    ctrl.computeControl(x0, 1)
    x_start = np.array([0.03, -0.02, 0.25, 0.05], np.float32)
    ctrl.computeFeedback(x_start)
    got = _gains_array(ctrl.getFeedbackState(), T, 2, 4)
    xt = ctrl.getTargetStateSeqs()[0].T.copy()
    un = ctrl.getControlSeqs()[0].T.copy()
    d = np.float32(damping)

    def f(x, u):
        x = np.asarray(x, np.float32)
        u = np.asarray(u, np.float32)
        return np.array([x[2], x[3], u[0] - d * x[2], u[1] - d * x[3]], np.float32)

    def analytic(x, u):
        A_ = np.zeros((4, 4))
        A_[0, 2] = A_[1, 3] = 1.0
        A_[2, 2] = A_[3, 3] = -float(d)
        B_ = np.zeros((4, 2))
        B_[2, 0] = B_[3, 1] = 1.0
        return A_, B_

    df = analytic if name == "di_quadratic" else (lambda x, u: oddp.numeric_grad(f, x, u))
    lo, hi = np.array([-2.0, -2.0], np.float32), np.array([2.0, 2.0], np.float32)
    ref = oddp.ddp_gains(f, df, x_start, xt, un, dt, Q, Q, R, 1, lo, hi)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    if name == "di_symplectic_quadratic":
        exact = oddp.ddp_gains(f, analytic, x_start, xt, un, dt, Q, Q, R, 1, lo, hi)
        assert np.abs(got - exact).max() <= 5e-2 * np.abs(exact).max()  # forward differences, not exact
    ctrl.close()


def test_feedback_needs_a_single_controller():
    from mppi_generic_vendor_gb300 import BatchedMPPIController, MPPIError

    ctrl = BatchedMPPIController(DoubleIntegratorDynamics(), DoubleIntegratorObstacleCost(),
                                 GaussianDistribution(std_dev=(0.5, 0.5)), [256, 256], [16, 16])
    with pytest.raises(MPPIError):
        ctrl.initFeedback()
    ctrl.close()
