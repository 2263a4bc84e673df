"""Shared parity checks of the updated control sequence against the oracle.

The update is a weighted sum, u_j = sum_k (w_k / eta) u_kj, followed by the Savitzky-Golay taps c = [-3, 12, 17, 12,
-3] / 35 and the clamp.  The engine sums in FP32 tile by tile, the oracle in FP64, so the rounding error of element j
is bounded by a small multiple of the magnitude of the terms it sums,

    A_j = sum_i |c_i| sum_k (w_k / eta) |u_k,j+i|     (A_0 = sum_k (w_k / eta) |u_k,0|, u_0 is not smoothed),

not of u_j itself, which can be near zero when the weighted samples cancel.  The check is element-wise:
|got_j - ref_j| <= rtol * A_j, with rtol = 1e-5; A_j >= |ref_j| always, and A_j = |ref_j| when the samples of an
element share its sign.  It also reports the plain element-wise relative error |got_j - ref_j| / |ref_j|.
"""
import numpy as np

import oracle

TAPS = np.array([-3.0, 12.0, 17.0, 12.0, -3.0]) / 35.0


def term_magnitude(weights, normalizer, samples, K, T, Cdim, smoothed=True):
    """A_j of the module docstring, float64 [T][C] (smoothed=False: the unsmoothed update, A_j = the inner sum)."""
    _, absout = oracle.weighted_mean(weights, np.float32(normalizer), samples, K, T, Cdim)
    a = absout.reshape(T, Cdim)
    if not smoothed:
        return a
    pad = np.concatenate([a[:1], a[:1], a, a[-1:], a[-1:]])
    out = np.zeros_like(a)
    for i, c in enumerate(TAPS):
        out += abs(c) * pad[i:i + T]
    out[0] = a[0]
    return out


def check_control(got_tc, ref, K, T, Cdim, rtol=1e-5, samples=None, smoothed=True):
    """Element-wise check of an updated control sequence (float [T][C]) against an oracle result dict (control,
    weights, normalizer, samples); returns (max error / A_j, median element-wise relative error)."""
    s = ref["samples"] if samples is None else samples
    A = term_magnitude(ref["weights"], ref["normalizer"], s, K, T, Cdim, smoothed=smoothed)
    got = np.asarray(got_tc, np.float64).reshape(T, Cdim)
    exp = np.asarray(ref["control"], np.float64).reshape(T, Cdim)
    err = np.abs(got - exp)
    ratio = err / np.maximum(A, 1e-30)
    assert np.all(err <= rtol * A), (float(ratio.max()), np.unravel_index(int(np.argmax(ratio)), ratio.shape))
    nz = np.abs(exp) > 0
    rel = float(np.median(err[nz] / np.abs(exp[nz]))) if nz.any() else 0.0
    return float(ratio.max()), rel


def solve_from_samples(model, dyn, cost, cparams, sampling, constraints, K, T, Cdim, S, x0, samples, control,
                       costmap=None, lambda_=None):
    """The oracle's update of one MPPI iteration (mppi_controller.cu:162-216, then smoothing and the clamp) on given
    constrained control samples (float [K][T][C]): rollout costs, weights, FP64 weighted mean, smoothing, clamp —
    the steps of oracle.compute_control after its sampler."""
    lam = cparams.lambda_ if lambda_ is None else lambda_
    u = np.ascontiguousarray(samples, np.float32).reshape(-1).copy()
    c64, u, _ = oracle.rollout(model, dyn, cost, x0, u, control, sampling, constraints, lam, cparams.alpha, K, T,
                               cparams.dt, costmap=costmap, state_dim=S)
    costs = c64.astype(np.float32)
    w, b, n = oracle.weights(costs, lambda_inv=np.float32(1.0) / np.float32(lam))
    mean, _ = oracle.weighted_mean(w, np.float32(n), u, K, T, Cdim)
    ctl = oracle.smooth(mean.astype(np.float32).reshape(T, Cdim))
    ctl = oracle.enforce_constraints(ctl, Cdim, constraints).reshape(T, Cdim)
    return dict(costs=costs, weights=w, baseline=b, normalizer=n, control=ctl, samples=u)
