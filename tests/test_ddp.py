"""The DDP feedback controller's solver (DDP::run, ddp/ddp.h:40-195, over the tracking costs of
ddp/ddp_tracking_costs.h) through mppi_ddp_feedback_gains, the handle-free entry point that runs the same host code as
mppi_compute_feedback: against the oracle's NumPy restatement for every built-in analytic model (analytic Jacobians
for the cart-pole, the double integrator and the kinematic bicycle, forward differences for the dynamic bicycle),
with the line search of several iterations, and for the linear double integrator against the textbook discrete
Riccati recursion.  No GPU is involved."""
import numpy as np
import pytest

import oracle
from oracle import ddp as oddp
from mppi_generic_vendor_gb300 import (BicycleDynamics, BicycleSlipDynamics, CartpoleDynamics, CartpoleSwingupCost,
                                       CostmapCost, DoubleIntegratorDynamics, DoubleIntegratorObstacleCost)
from mppi_generic_vendor_gb300 import _abi as A
from _ddp import engine_gains


def _problem(model, dyn, cost, H, dt, seed, u_scale, x0):
    """A nominal trajectory (states of a rollout of random controls) and a perturbed start state."""
    rng = np.random.default_rng(seed)
    f, _ = oddp.model_functions(model, dyn, cost)
    S = len(x0)
    un = (rng.standard_normal((H, len(u_scale))) * u_scale).astype(np.float32)
    xt = np.zeros((H, S), np.float32)
    xt[0] = x0
    for t in range(1, H):
        xt[t] = (xt[t - 1] + f(xt[t - 1], un[t - 1]) * np.float32(dt)).astype(np.float32)
    x_start = (xt[0] + 0.05 * rng.standard_normal(S)).astype(np.float32)
    return x_start, xt, un


CASES = [
    (A.MODEL_CARTPOLE, lambda: CartpoleDynamics().getParams(), lambda: CartpoleSwingupCost().getParams(),
     [2.0], [0.1, 0.0, 3.0, 0.0]),
    (A.MODEL_DOUBLE_INTEGRATOR, lambda: DoubleIntegratorDynamics().getParams(),
     lambda: DoubleIntegratorObstacleCost().getParams(), [0.5, 0.5], [1.0, -1.0, 0.2, 0.1]),
    (A.MODEL_BICYCLE_COSTMAP, lambda: BicycleDynamics().getParams(), lambda: CostmapCost().getParams(), [1.0, 0.2],
     [1.0, 2.0, 0.3, 5.0]),
    (A.MODEL_BICYCLE_SLIP, lambda: BicycleSlipDynamics().getParams(), lambda: CostmapCost().getParams(),
     [0.3, 0.3], [1.0, 2.0, 0.3, 6.0, 0.1, 0.05, 0.0]),
]


@pytest.mark.parametrize("model,dyn_f,cost_f,u_scale,x0", CASES, ids=["cartpole", "di", "bicycle", "slip"])
@pytest.mark.parametrize("iterations", [1, 3])
def test_gains_match_oracle(model, dyn_f, cost_f, u_scale, x0, iterations):
    dyn, cost = dyn_f(), cost_f()
    H, dt = 40, 0.02
    x_start, xt, un = _problem(model, dyn, cost, H, dt, 3, np.array(u_scale, np.float32),
                               np.array(x0, np.float32))
    S, Cd = xt.shape[1], un.shape[1]
    rng = np.random.default_rng(11)
    Q = np.diag(rng.uniform(0.5, 5.0, S)).astype(np.float32)
    Qf = np.diag(rng.uniform(5.0, 20.0, S)).astype(np.float32)
    R = np.diag(rng.uniform(0.05, 0.5, Cd)).astype(np.float32)
    lo, hi = -3.0 * np.ones(Cd, np.float32), 3.0 * np.ones(Cd, np.float32)
    st, got = engine_gains(model, dyn, x_start, xt, un, dt, Q, Qf, R, iterations, lo, hi)
    assert st == A.MPPI_OK, A.lib().mppi_last_error_string()
    f, df = oddp.model_functions(model, dyn, cost)
    ref = oddp.ddp_gains(f, df, x_start, xt, un, dt, Q, Qf, R, iterations, lo, hi)
    assert np.all(got[-1] == 0.0)
    scale = np.abs(ref).max()
    assert scale > 0
    # Forward differences (the dynamic bicycle) are exact only on a shared trajectory: after the first iteration the
    # line-search rollouts of the two float64 solvers can differ by an ulp, and a difference quotient with
    # h = 3.5e-4 |x| turns that into about 3e-4 of a Jacobian entry, so later iterations agree to about 5e-2.
    tol = 5e-2 if (model == A.MODEL_BICYCLE_SLIP and iterations > 1) else 1e-5
    assert np.abs(got - ref).max() <= tol * scale, np.abs(got - ref).max() / scale


def test_double_integrator_gains_are_the_riccati_solution():
    """For linear dynamics and a quadratic cost one DDP iteration is exact: the gains equal the time-varying LQR of
    x_{k+1} = Ad x_k + Bd u_k with stage cost dt (x'Qx + u'Ru) and terminal x'Qf x."""
    dyn, cost = DoubleIntegratorDynamics().getParams(), DoubleIntegratorObstacleCost().getParams()
    H, dt = 60, 0.05
    x_start, xt, un = _problem(A.MODEL_DOUBLE_INTEGRATOR, dyn, cost, H, dt, 5, np.array([0.4, 0.4], np.float32),
                               np.array([0.5, 0.5, 0.0, 0.0], np.float32))
    Q = np.diag([4.0, 4.0, 1.0, 1.0]).astype(np.float32)
    Qf = np.diag([30.0, 30.0, 5.0, 5.0]).astype(np.float32)
    R = np.diag([0.2, 0.3]).astype(np.float32)
    st, got = engine_gains(A.MODEL_DOUBLE_INTEGRATOR, dyn, x_start, xt, un, dt, Q, Qf, R)
    assert st == A.MPPI_OK
    Ad = np.eye(4)
    Ad[0, 2] = Ad[1, 3] = dt
    Bd = np.zeros((4, 2))
    Bd[2, 0] = Bd[3, 1] = dt
    P = Qf.astype(np.float64)
    K = np.zeros((H, 2, 4))
    for k in range(H - 2, -1, -1):
        G = R * dt + Bd.T @ P @ Bd
        K[k] = -np.linalg.solve(G, Bd.T @ P @ Ad)
        P = Q * dt + Ad.T @ P @ Ad + Ad.T @ P @ Bd @ K[k]
        P = 0.5 * (P + P.T)
    assert np.allclose(got, K, rtol=1e-5, atol=1e-6 * np.abs(K).max())


def test_weight_layout_is_column_major():
    """A non-symmetric R changes the gains by its transpose: the weights are read column-major."""
    dyn, cost = DoubleIntegratorDynamics().getParams(), DoubleIntegratorObstacleCost().getParams()
    H, dt = 20, 0.05
    x_start, xt, un = _problem(A.MODEL_DOUBLE_INTEGRATOR, dyn, cost, H, dt, 9, np.array([0.4, 0.4], np.float32),
                               np.array([0.5, 0.5, 0.0, 0.0], np.float32))
    R = np.array([[1.0, 0.3], [0.0, 1.0]], np.float32)  # quu stays positive definite either way
    f, df = oddp.model_functions(A.MODEL_DOUBLE_INTEGRATOR, dyn, cost)
    st, got = engine_gains(A.MODEL_DOUBLE_INTEGRATOR, dyn, x_start, xt, un, dt, None, None, R)
    assert st == A.MPPI_OK
    ref = oddp.ddp_gains(f, df, x_start, xt, un, dt, np.eye(4), np.eye(4), R)
    ref_t = oddp.ddp_gains(f, df, x_start, xt, un, dt, np.eye(4), np.eye(4), R.T)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    assert np.abs(got - ref_t).max() > 1e-3 * np.abs(ref).max()


def test_rejections():
    dyn, cost = DoubleIntegratorDynamics().getParams(), DoubleIntegratorObstacleCost().getParams()
    H, dt = 10, 0.05
    x_start, xt, un = _problem(A.MODEL_DOUBLE_INTEGRATOR, dyn, cost, H, dt, 1, np.array([0.4, 0.4], np.float32),
                               np.array([0.5, 0.5, 0.0, 0.0], np.float32))
    st, _ = engine_gains(A.MODEL_DOUBLE_INTEGRATOR, dyn, x_start, xt, un, dt, R=-np.eye(2, dtype=np.float32))
    assert st == A.MPPI_EINVAL and b"positive definite" in A.lib().mppi_last_error_string()
    st, _ = engine_gains(A.MODEL_DOUBLE_INTEGRATOR, dyn, x_start[:], xt[:1], un[:1], dt)
    assert st == A.MPPI_EINVAL
    st, _ = engine_gains(A.MODEL_DOUBLE_INTEGRATOR, dyn, x_start, xt, un, dt, iterations=0)
    assert st == A.MPPI_EINVAL
    st, _ = engine_gains(A.MODEL_BICYCLE_SLIP_MLP, BicycleSlipDynamics().getParams(), np.zeros(7), np.zeros((10, 7)),
                         np.zeros((10, 2)), dt)
    assert st == A.MPPI_EUNSUPPORTED
