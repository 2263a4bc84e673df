"""CPU oracle for the GB300 MPPI engine — TEST INFRASTRUCTURE ONLY.

A restatement of MPPI-Generic's plain MPPI path in C++ (mppi_oracle.cpp), loaded through ctypes.  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use it, and only as the checker or the timed
CPU reference; the engine never calls it.  Parameter blocks are passed as ctypes structures (or anything exposing the
buffer protocol) laid out as in include/mppi_gb.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB = ORACLE_DIR / "_build" / "libmppi_oracle.so"
_lib = None

_P = C.c_void_p
_FP = C.POINTER(C.c_float)
_DP = C.POINTER(C.c_double)
_U32P = C.POINTER(C.c_uint32)

_SIGS = [
    ("orc_sincosf", None, [_FP, _FP, _FP, C.c_size_t]),
    ("orc_normalize_angle", C.c_float, [C.c_float]),
    ("orc_set_trig_mode", None, [C.c_int]),
    ("orc_get_trig_mode", C.c_int, []),
    ("orc_philox4x32_10", None, [_U32P, _U32P, _U32P]),
    ("orc_gaussian_rewrite", None, [_FP, _FP, _FP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, _FP]),
    ("orc_enforce_constraints", None, [_FP, C.c_size_t, C.c_int, _P]),
    ("orc_dynamics_deriv", C.c_int, [C.c_int, _P, _P, _DP, _DP, _DP, C.c_int]),
    ("orc_rollout", C.c_int, [C.c_int, _P, _P, _FP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _FP, _FP, _FP,
                              _P, _P, C.c_float, C.c_float, C.c_int, C.c_int, C.c_float, _DP, _DP, C.c_int,
                              C.c_int]),
    ("orc_weights", None, [_FP, C.c_int, C.c_float, _FP, _FP, _DP]),
    ("orc_tsallis", None, [_FP, C.c_int, C.c_float, C.c_float, C.c_float, _FP]),
    ("orc_weighted_mean", None, [_FP, C.c_float, _FP, C.c_int, C.c_int, C.c_int, _DP, _DP]),
    ("orc_smooth", None, [_FP, C.c_int, C.c_int]),
    ("orc_slide", None, [_FP, C.c_int, C.c_int, C.c_int, _FP, _FP]),
    ("orc_colored_scales", None, [C.c_int, C.c_int, _FP, C.c_float, _FP, _FP]),
    ("orc_colored_noise", None, [_FP, C.c_int, C.c_int, C.c_int, _FP, C.c_float, C.c_float, C.c_int, _FP,
                                 C.c_int]),
    ("orc_rmppi_rollout", C.c_int, [C.c_int, _P, _P, _FP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _FP,
                                    _FP, _FP, _FP, _FP, _FP, _FP, _P, _P, C.c_float, C.c_float, C.c_float, C.c_int,
                                    C.c_int, C.c_float, _FP, _FP, C.c_int]),
    ("orc_rmppi_eval", C.c_int, [C.c_int, _P, _P, _FP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _FP,
                                 C.POINTER(C.c_int), C.c_int, C.c_int, _FP, _FP, _P, _P, C.c_float, C.c_float, C.c_int,
                                 C.c_int, C.c_float, _FP]),
    ("orc_compute_control", C.c_int, [C.c_int, _P, _P, _FP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _P,
                                      _P, _P, C.c_int, C.c_int, _FP, _FP, C.c_int, C.c_int, _FP, _FP, _FP, _FP,
                                      _FP, _DP, _FP, C.c_int]),
]


def build(force: bool = False) -> Path:
    """Compile the oracle with its Makefile (g++, no CUDA)."""
    args = ["make", "-s", "-C", str(ORACLE_DIR)]
    if force:
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "clean"], check=True)
    subprocess.run(args, check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        for name, res, args in _SIGS:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_FP)


def _ptr(struct):
    return None if struct is None else C.cast(C.byref(struct), C.c_void_p)


def threads_default() -> int:
    return max(1, os.cpu_count() or 1)


def sincosf(x):
    x = _f32(x).reshape(-1)
    s = np.empty_like(x)
    c = np.empty_like(x)
    lib().orc_sincosf(_fp(x), _fp(s), _fp(c), x.size)
    return s, c


class libm_trig:
    """Context manager: the float oracle evaluates sine / cosine with libm sinf / cosf (the reference's host twins,
    e.g. cartpole_dynamics.cu:48-53) instead of the engine's own sincos_f."""

    def __enter__(self):
        lib().orc_set_trig_mode(1)
        return self

    def __exit__(self, *exc):
        lib().orc_set_trig_mode(0)
        return False


def normalize_angle(a: float) -> float:
    return lib().orc_normalize_angle(float(a))


def philox4x32_10(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def gaussian_rewrite(eps, mean, std_dev, K, T, Cdim, stride, decay_pow=1.0, pure_pct=0.01):
    e = _f32(eps).reshape(-1)
    m = _f32(mean).reshape(-1)
    s = _f32(std_dev).reshape(-1)
    out = np.empty_like(e)
    lib().orc_gaussian_rewrite(_fp(e), _fp(m), _fp(s), K, T, Cdim, stride, decay_pow, pure_pct, _fp(out))
    return out


def enforce_constraints(u, Cdim, constraints):
    u = _f32(u).copy().reshape(-1)
    lib().orc_enforce_constraints(_fp(u), u.size // Cdim, Cdim, _ptr(constraints))
    return u


def dynamics_deriv(model, dyn, cost, x, u, fp64=True):
    x = np.ascontiguousarray(x, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    xd = np.zeros(8, dtype=np.float64)
    lib().orc_dynamics_deriv(model, _ptr(dyn), _ptr(cost), x.ctypes.data_as(_DP), u.ctypes.data_as(_DP),
                             xd.ctypes.data_as(_DP), int(fp64))
    return xd[: x.size]


def rollout(model, dyn, cost, x0, controls, mean, sampling, constraints, lambda_, alpha, K, T, dt, costmap=None,
            threads=None, fp64=False, want_traj=False, state_dim=4):
    """Returns (costs float64[K], constrained controls float32, trajectory or None)."""
    u = _f32(controls).copy().reshape(-1)
    x0 = _f32(x0).reshape(-1)
    mean = _f32(mean).reshape(-1)
    costs = np.empty(K, dtype=np.float64)
    traj = np.empty(K * T * state_dim, dtype=np.float64) if want_traj else None
    if costmap is not None:
        data, res, (ox, oy) = costmap
        data = _f32(data)
        mp, mw, mh = _fp(data), data.shape[1], data.shape[0]
    else:
        data, mp, mw, mh, res, ox, oy = None, None, 0, 0, 1.0, 0.0, 0.0
    rc = lib().orc_rollout(model, _ptr(dyn), _ptr(cost), mp, mw, mh, res, ox, oy, _fp(x0), _fp(u), _fp(mean),
                           _ptr(sampling), _ptr(constraints), lambda_, alpha, K, T, dt, costs.ctypes.data_as(_DP),
                           None if traj is None else traj.ctypes.data_as(_DP), threads or threads_default(),
                           int(fp64))
    if rc != 0:
        raise ValueError(f"oracle has no model {model}")
    return costs, u, traj


def weights(costs, lambda_=None, lambda_inv=None):
    """Baseline, exp weights and normaliser; give lambda_ or lambda_inv (float32 1/lambda as the engine uses)."""
    c = _f32(costs)
    w = np.empty_like(c)
    b = C.c_float()
    n = C.c_double()
    linv = np.float32(lambda_inv) if lambda_inv is not None else np.float32(1.0) / np.float32(lambda_)
    lib().orc_weights(_fp(c), c.size, float(linv), _fp(w), C.byref(b), C.byref(n))
    return w, b.value, n.value


def tsallis(costs, gamma, r, baseline):
    """TsallisTransform (mppi_common.cu:1004-1021): weights (1 - d / gamma)^(1 / (r - 1)) for d = c - baseline <
    gamma, else 0."""
    c = _f32(costs)
    w = np.empty_like(c)
    lib().orc_tsallis(_fp(c), c.size, float(gamma), float(r), float(baseline), _fp(w))
    return w


def weighted_mean(w, normalizer, controls, K, T, Cdim):
    w = _f32(w)
    u = _f32(controls).reshape(-1)
    out = np.empty(T * Cdim, dtype=np.float64)
    absout = np.empty(T * Cdim, dtype=np.float64)
    lib().orc_weighted_mean(_fp(w), float(normalizer), _fp(u), K, T, Cdim, out.ctypes.data_as(_DP),
                            absout.ctypes.data_as(_DP))
    return out, absout


def smooth(u_tc):
    u = _f32(u_tc).copy()
    T, Cdim = u.shape
    lib().orc_smooth(_fp(u), T, Cdim)
    return u


def slide(u_tc, steps, scale, zero):
    u = _f32(u_tc).copy()
    T, Cdim = u.shape
    sc = _f32(scale)
    z = _f32(zero)
    lib().orc_slide(_fp(u), T, Cdim, steps, _fp(sc), _fp(z))
    return u


def colored_scales(T, Cdim, exponents, fmin=0.0):
    e = _f32(exponents)
    s = np.empty((T + 1) * Cdim, dtype=np.float32)
    sg = np.empty(Cdim, dtype=np.float32)
    lib().orc_colored_scales(T, Cdim, _fp(e), fmin, _fp(s), _fp(sg))
    return s.reshape(T + 1, Cdim), sg


def colored_noise(spectrum, K, T, Cdim, exponents, fmin=0.0, decay=0.97, offset_t=1, threads=None):
    sp = _f32(spectrum).reshape(-1)
    e = _f32(exponents)
    out = np.empty(K * T * Cdim, dtype=np.float32)
    lib().orc_colored_noise(_fp(sp), K, T, Cdim, _fp(e), fmin, decay, offset_t, _fp(out),
                            threads or threads_default())
    return out


def compute_control(model, dyn, cost, cparams, sampling, constraints, K, T, Cdim, S, x0, eps, control, stride=1,
                    same_noise_each_iter=True, costmap=None, threads=None):
    """One VanillaMPPIController::computeControl on the CPU; returns a dict of the results."""
    control = _f32(control).copy().reshape(-1)
    x0 = _f32(x0).reshape(-1)
    eps = _f32(eps).reshape(-1)
    costs = np.empty(K, dtype=np.float32)
    w = np.empty(K, dtype=np.float32)
    samples = np.empty(K * T * Cdim, dtype=np.float32)
    state = np.empty(T * S, dtype=np.float32)
    b = C.c_float()
    n = C.c_double()
    if costmap is not None:
        data, res, (ox, oy) = costmap
        data = _f32(data)
        mp, mw, mh = _fp(data), data.shape[1], data.shape[0]
    else:
        mp, mw, mh, res, ox, oy = None, 0, 0, 1.0, 0.0, 0.0
    rc = lib().orc_compute_control(model, _ptr(dyn), _ptr(cost), mp, mw, mh, res, ox, oy, _ptr(cparams),
                                   _ptr(sampling), _ptr(constraints), K, T, _fp(x0), _fp(eps),
                                   int(same_noise_each_iter), stride, _fp(control), _fp(costs), _fp(w),
                                   _fp(samples), C.byref(b), C.byref(n), _fp(state), threads or threads_default())
    if rc != 0:
        raise ValueError(f"oracle has no model {model}")
    return dict(control=control.reshape(T, Cdim), costs=costs, weights=w, samples=samples, baseline=b.value,
                normalizer=n.value, state_seq=state.reshape(T, S))


# ------------------------------------------------------------------------------------------------ MLP surrogate
def _mlp_sigs():
    L = lib()
    L.orc_mlp_num_params.restype = C.c_int
    L.orc_mlp_forward.argtypes = [_FP, _FP, C.c_int, _DP]
    L.orc_mlp_loss_grad.restype = C.c_double
    L.orc_mlp_loss_grad.argtypes = [_DP, _FP, _FP, C.c_int, _DP]
    return L


def mlp_num_params() -> int:
    return _mlp_sigs().orc_mlp_num_params()


def mlp_forward(params, X):
    L = _mlp_sigs()
    p = _f32(params)
    X = _f32(X).reshape(-1, 9)
    Y = np.empty((X.shape[0], 5), dtype=np.float64)
    L.orc_mlp_forward(_fp(p), _fp(X), X.shape[0], Y.ctypes.data_as(_DP))
    return Y


def mlp_loss_grad(params, X, Y):
    """MSE loss and its gradient in FP64 by hand back-propagation (params in float64)."""
    L = _mlp_sigs()
    p = np.ascontiguousarray(params, dtype=np.float64)
    X = _f32(X).reshape(-1, 9)
    Y = _f32(Y).reshape(-1, 5)
    g = np.empty_like(p)
    loss = L.orc_mlp_loss_grad(p.ctypes.data_as(_DP), _fp(X), _fp(Y), X.shape[0], g.ctypes.data_as(_DP))
    return loss, g


def set_mlp(params):
    """Surrogate parameters (network + normalisation, 5153 floats) for the MLP bicycle model
    (model id 5) in rollout / compute_control / dynamics_deriv."""
    p = _f32(params).reshape(-1)
    if p.size != 5153:
        raise ValueError("surrogate parameter vector must hold 5153 floats")
    L = lib()
    L.orc_set_mlp.argtypes = [_FP]
    L.orc_set_mlp(_fp(p))


def tube_compute_control(model, dyn, cost, cparams, sampling, constraints, K, T, Cdim, S, x_actual, nominal_x0, eps,
                         control, stride=1, costmap=None, threads=None):
    """One TubeMPPIController::computeControl on the CPU.  eps: [2][K][T][C] standard normals (actual, nominal);
    control: [2][T][C] (actual, nominal) in; returns a dict with both updated sequences, the nominal state after the
    call, costs / weights / samples of both distributions, baselines, normalisers, nominal_used and both state
    trajectories."""
    ctl = _f32(control).copy().reshape(-1)
    xa = _f32(x_actual).reshape(-1)
    xn = _f32(nominal_x0).copy().reshape(-1)
    e = _f32(eps).reshape(-1)
    costs = np.empty(2 * K, np.float32)
    w = np.empty(2 * K, np.float32)
    samples = np.empty(2 * K * T * Cdim, np.float32)
    b = np.empty(2, np.float32)
    n = np.empty(2, np.float64)
    used = C.c_int()
    states = np.empty(2 * T * S, np.float32)
    if costmap is not None:
        data, res, (ox, oy) = costmap
        data = _f32(data)
        mp, mw, mh = _fp(data), data.shape[1], data.shape[0]
    else:
        mp, mw, mh, res, ox, oy = None, 0, 0, 1.0, 0.0, 0.0
    L = lib()
    L.orc_tube_compute_control.restype = C.c_int
    rc = L.orc_tube_compute_control(model, _ptr(dyn), _ptr(cost), mp, mw, mh, C.c_float(res), C.c_float(ox),
                                    C.c_float(oy), _ptr(cparams), _ptr(sampling), _ptr(constraints), K, T, _fp(xa),
                                    _fp(xn), _fp(e), stride, _fp(ctl), _fp(costs), _fp(w), _fp(samples), _fp(b),
                                    n.ctypes.data_as(_DP), C.byref(used), _fp(states), threads or threads_default())
    if rc != 0:
        raise ValueError(f"oracle has no model {model}")
    return dict(control=ctl.reshape(2, T, Cdim), nominal_x0=xn, costs=costs.reshape(2, K), weights=w.reshape(2, K),
                samples=samples.reshape(2, K * T * Cdim), baselines=b, normalizers=n, nominal_used=used.value,
                state_seq=states.reshape(2, T, S))


def _map_args(costmap):
    if costmap is not None:
        data, res, (ox, oy) = costmap
        data = _f32(data)
        return data, (_fp(data), data.shape[1], data.shape[0], res, ox, oy)
    return None, (None, 0, 0, 1.0, 0.0, 0.0)


def rmppi_rollout(model, dyn, cost, x0_nom, x0_real, samples_nom, samples_real, mean_nom, mean_real, gains, sampling,
                  constraints, lambda_, alpha, threshold, K, T, dt, costmap=None, threads=None):
    """rolloutRMPPIKernel restated: returns (nominal costs, real costs, constrained nominal samples, constrained real
    samples with feedback), all float32; gains are [T][C*S] (column-major per step)."""
    un = _f32(samples_nom).copy().reshape(-1)
    ur = _f32(samples_real).copy().reshape(-1)
    cn = np.empty(K, np.float32)
    cr = np.empty(K, np.float32)
    keep, m = _map_args(costmap)
    args = [_f32(a).reshape(-1) for a in (x0_nom, x0_real, mean_nom, mean_real, gains)]
    rc = lib().orc_rmppi_rollout(model, _ptr(dyn), _ptr(cost), *m, _fp(args[0]), _fp(args[1]), _fp(un), _fp(ur),
                                 _fp(args[2]), _fp(args[3]), _fp(args[4]), _ptr(sampling), _ptr(constraints), lambda_,
                                 alpha, threshold, K, T, dt, _fp(cn), _fp(cr), threads or threads_default())
    if rc != 0:
        raise ValueError(f"oracle has no R-MPPI model {model}")
    return cn, cr, un, ur


def rmppi_eval(model, dyn, cost, cand_states, cand_strides, per_cand, samples, mean, sampling, constraints, lambda_,
               alpha, K, T, dt, costmap=None):
    """initEvalKernel restated: costs float32[num_cand * per_cand]."""
    cs = _f32(cand_states).reshape(-1)
    st = np.ascontiguousarray(cand_strides, dtype=np.int32)
    smp = _f32(samples).reshape(-1)
    mn = _f32(mean).reshape(-1)
    out = np.empty(st.size * per_cand, np.float32)
    keep, m = _map_args(costmap)
    rc = lib().orc_rmppi_eval(model, _ptr(dyn), _ptr(cost), *m, _fp(cs), st.ctypes.data_as(C.POINTER(C.c_int)),
                              st.size, per_cand, _fp(smp), _fp(mn), _ptr(sampling), _ptr(constraints), lambda_, alpha,
                              K, T, dt, _fp(out))
    if rc != 0:
        raise ValueError(f"oracle has no R-MPPI model {model}")
    return out


def step_state(model, dyn, cost, x, u, dt):
    """x after one Dynamics::step with control u (no constraint), in float."""
    xs = _f32(x).copy().reshape(-1)
    us = _f32(u).reshape(-1)
    L = lib()
    L.orc_step_state.restype = C.c_int
    if L.orc_step_state(model, _ptr(dyn), _ptr(cost), _fp(us), C.c_float(dt), _fp(xs)) != 0:
        raise ValueError(f"oracle has no model {model}")
    return xs
