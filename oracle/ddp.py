"""DDP tracking feedback restated in NumPy — TEST INFRASTRUCTURE ONLY (the checker of the engine's feedback controller).

Follows the reference's ancillary controller:
  * DDP::run (include/mppi/ddp/ddp.h:40-195): Euler rollout of the nominal controls (controls 0 .. H-3 clamped),
    Jacobians Phi = I + A dt, B dt, backward pass with qx, qu, qux, qxx, quu, K = -quu^-1 qux, k = -quu^-1 qu,
    symmetrised Vxx, then the forward pass with the halving line search;
  * TrackingCostDDP / TrackingTerminalCost (include/mppi/ddp/ddp_tracking_costs.h:8-128): cost (x-x*)'Q(x-x*) +
    (u-u*)'R(u-u*), gradient (Q (x-x*), R (u-u*)), Hessian diag(Q, R); terminal (x-xf)'Qf(x-xf);
  * ModelWrapperDDP::f / df (include/mppi/ddp/ddp_model_wrapper.h:66-94): xdot of the model's step, analytic
    computeGrad where the model has one (CartpoleDynamics::computeGrad, cartpole_dynamics.cu:10-45;
    DoubleIntegratorDynamics::computeGrad, di_dynamics.cu:24-34), else Eigen's forward-difference NumericalDiff.
The dynamics are the oracle's FP32 model (``oracle.dynamics_deriv``); the linear algebra is float64.
"""
from __future__ import annotations

import numpy as np

from . import dynamics_deriv

MODEL_CARTPOLE, MODEL_DOUBLE_INTEGRATOR, MODEL_BICYCLE_COSTMAP, MODEL_BICYCLE_SLIP = 1, 2, 3, 4


def cartpole_grad(p, x, u):
    """CartpoleDynamics::computeGrad (cartpole_dynamics.cu:10-45) in float64, term for term."""
    mc, mp, lp, g = float(p.cart_mass), float(p.pole_mass), float(p.pole_length), float(p.gravity)
    th, td, f = float(x[2]), float(x[3]), float(u[0])
    s, c = np.sin(th), np.cos(th)
    A = np.zeros((4, 4))
    B = np.zeros((4, 1))
    A[0, 1] = 1.0
    A[1, 2] = ((mp * c * (lp * td ** 2 + g * c) - g * mp * s ** 2) / (mc + mp * s ** 2)
               - (2 * mp * c * s * (f + mp * s * (lp * td ** 2 + g * c))) / (mc + mp * s ** 2) ** 2)
    A[1, 3] = (2 * lp * mp * td * s) / (mc + mp * s ** 2)
    A[2, 3] = 1.0
    A[3, 2] = ((f * s - g * c * (mp + mc) - lp * mp * td ** 2 * c ** 2 + lp * mp * td ** 2 * s ** 2)
               / (lp * (mc + mp * s ** 2))
               + (2 * mp * c * s * (lp * mp * c * s * td ** 2 + f * c + g * s * (mp + mc)))
               / (lp * (mc + mp * s ** 2)) ** 2)
    A[3, 3] = -(2 * mp * td * c * s) / (mc + mp * s ** 2)
    B[1, 0] = 1 / (mc + mp * s ** 2)
    B[3, 0] = -c / (lp * (mc + mp * s ** 2))
    return A, B


def double_integrator_grad(p, x, u):
    """DoubleIntegratorDynamics::computeGrad (di_dynamics.cu:24-34)."""
    A = np.zeros((4, 4))
    B = np.zeros((4, 2))
    A[0, 2] = A[1, 3] = 1.0
    B[2, 0] = B[3, 1] = 1.0
    return A, B


def bicycle_grad(p, x, u):
    """Derivatives of the kinematic bicycle (x, y, yaw, v; accel, steer): xdot = v cos yaw, ydot = v sin yaw,
    yawdot = v tan(steer) / L, vdot = accel (no reference counterpart)."""
    yaw, v, steer, L = float(x[2]), float(x[3]), float(u[1]), float(p.wheelbase)
    A = np.zeros((4, 4))
    B = np.zeros((4, 2))
    A[0, 2], A[0, 3] = -v * np.sin(yaw), np.cos(yaw)
    A[1, 2], A[1, 3] = v * np.cos(yaw), np.sin(yaw)
    A[2, 3] = np.tan(steer) / L
    B[2, 1] = v / (L * np.cos(steer) ** 2)
    B[3, 0] = 1.0
    return A, B


ANALYTIC = {MODEL_CARTPOLE: cartpole_grad, MODEL_DOUBLE_INTEGRATOR: double_integrator_grad,
            MODEL_BICYCLE_COSTMAP: bicycle_grad}


def numeric_grad(f, x, u):
    """Eigen NumericalDiff, Forward mode with epsfcn 0 (ddp_dynamics.h:96-101), in float32: h_j = sqrt(eps) |v_j|
    (sqrt(eps) where v_j = 0), column j = (f(v + h_j e_j) - f(v)) / h_j."""
    S, Cd = len(x), len(u)
    v = np.concatenate([np.asarray(x, np.float32), np.asarray(u, np.float32)])
    eps = np.sqrt(np.float32(1.1920929e-7))
    f0 = f(v[:S], v[S:])
    J = np.zeros((S, S + Cd))
    for j in range(S + Cd):
        h = np.float32(eps * np.float32(abs(v[j])))
        if h == 0:
            h = eps
        w = v.copy()
        w[j] = np.float32(v[j] + h)
        J[:, j] = ((f(w[:S], w[S:]) - f0) / h).astype(np.float32)
    return J[:, :S], J[:, S:]


def model_functions(model, dyn, cost):
    """(f, df) of a built-in model: f in float32 through the oracle's model, df analytic or numeric."""
    def f(x, u):
        return dynamics_deriv(model, dyn, cost, np.asarray(x, np.float64), np.asarray(u, np.float64),
                              fp64=False).astype(np.float32)

    if model in ANALYTIC:
        grad = ANALYTIC[model]
        return f, lambda x, u: grad(dyn, x, u)
    return f, lambda x, u: numeric_grad(f, x, u)


def ddp_gains(f, df, x0, x_target, u_nom, dt, Q, Qf, R, iterations=1, u_min=None, u_max=None):
    """DDP::run for the tracking cost.  x_target (H, S), u_nom (H, C); returns the gains (H, C, S) (K_{H-1} = 0)."""
    x_target = np.asarray(x_target, np.float32)
    u_nom = np.asarray(u_nom, np.float32)
    H, S = x_target.shape
    Cd = u_nom.shape[1]
    Q, Qf, R = (np.asarray(m, np.float64) for m in (Q, Qf, R))
    lo = np.full(Cd, -np.inf, np.float32) if u_min is None else np.asarray(u_min, np.float32)
    hi = np.full(Cd, np.inf, np.float32) if u_max is None else np.asarray(u_max, np.float32)
    f32 = np.float32(dt)

    def euler(x, u):
        return (x + f(x, u) * f32).astype(np.float32)

    x = np.zeros((H, S), np.float32)
    u = u_nom.copy()
    x[0] = np.asarray(x0, np.float32)
    for i in range(1, H):
        if i < H - 1:
            u[i - 1] = np.fmax(np.fmin(u[i - 1], hi), lo)
        x[i] = euler(x[i - 1], u[i - 1])

    def cost(xk, uk, k):
        dx = xk.astype(np.float64) - x_target[k]
        du = uk.astype(np.float64) - u_nom[k]
        return dx @ Q @ dx + du @ R @ du

    K = np.zeros((H, Cd, S))
    kff = np.zeros((H, Cd))
    prev = None
    xf = x_target[H - 1].astype(np.float64)
    for it in range(iterations):
        Phi, Bd = [], []
        for k in range(H):
            A, B = df(x[k], u[k])
            Phi.append(np.eye(S) + np.asarray(A, np.float64) * dt)
            Bd.append(np.asarray(B, np.float64) * dt)
        Vxx = 0.5 * (Qf + Qf.T)
        Vx = Qf @ (x[H - 1].astype(np.float64) - xf)
        V_term = float((x[H - 1].astype(np.float64) - xf) @ Vx)
        for k in range(H - 2, -1, -1):
            P, B = Phi[k], Bd[k]
            lx = Q @ (x[k].astype(np.float64) - x_target[k])
            lu = R @ (u[k].astype(np.float64) - u_nom[k])
            qx = lx * dt + P.T @ Vx
            qu = lu * dt + B.T @ Vx
            qux = B.T @ Vxx @ P
            qxx = Q * dt + P.T @ Vxx @ P
            quu = R * dt + B.T @ Vxx @ B
            # Eigen's LDLT reads the lower triangle only (ddp.h:130-134)
            quu = np.tril(quu) + np.tril(quu, -1).T
            K[k] = np.linalg.solve(quu, -qux)
            kff[k] = np.linalg.solve(quu, -qu)
            nV = qxx + qux.T @ K[k]
            Vxx = 0.5 * (nV + nV.T)
            Vx = qx + qux.T @ kff[k]
        alpha = 1.0
        while True:
            xn = np.zeros_like(x)
            un = np.zeros_like(u)
            xn[0] = x[0]
            c = np.zeros(H)
            for k in range(H - 1):
                v = u[k].astype(np.float64) + alpha * kff[k] + K[k] @ (xn[k].astype(np.float64) - x[k])
                un[k] = np.fmax(np.fmin(v.astype(np.float32), hi), lo)
                xn[k + 1] = euler(xn[k], un[k])
                c[k] = cost(xn[k], un[k], k) * dt
            c[H - 1] = V_term
            if it == 0 or alpha < 1e-4 or c.sum() <= prev.sum():
                x, u, prev = xn, un, c
                break
            alpha *= 0.5
    return K.astype(np.float32)
