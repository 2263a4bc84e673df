"""Pins of the CPU oracle against the reference's own known answers (no GPU).

The oracle is the checker for every GPU parity test, so it is itself checked here against: the Philox4x32-10
known-answer vectors of its published definition, the smoothing / slide / equilibrium known answers of the
reference's tests, the normexp and weighted-reduction recipes of the reference's kernel tests, and the reference's
NumPy colored-noise generator run with the same normals.
"""
import math

import numpy as np
import pytest

import oracle
from mppi_generic_vendor_gb300 import _abi as A


def ulp(x):
    return np.spacing(np.abs(np.float32(x))).astype(np.float64)


def test_philox_known_answers():
    # Random123 kat_vectors for philox4x32_10 (Salmon et al., SC 2011)
    assert oracle.philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox4x32_10([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                                          0x6D5451FD]
    assert oracle.philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_sincos_accuracy():
    rng = np.random.default_rng(3)
    x = np.concatenate([np.linspace(-np.pi, np.pi, 200001), rng.uniform(-200, 200, 200000),
                        rng.uniform(-2e4, 2e4, 20000)]).astype(np.float32)
    s, c = oracle.sincosf(x)
    xs = x.astype(np.float64)
    es = np.abs(s - np.sin(xs)) / np.maximum(ulp(np.sin(xs)), 2.0 ** -149)
    ec = np.abs(c - np.cos(xs)) / np.maximum(ulp(np.cos(xs)), 2.0 ** -149)
    # absolute error bound near the zeros, 2-ulp bound elsewhere
    ok_s = (es <= 2.0) | (np.abs(s - np.sin(xs)) < 2e-9)
    ok_c = (ec <= 2.0) | (np.abs(c - np.cos(xs)) < 2e-9)
    assert ok_s.all() and ok_c.all(), (es.max(), ec.max())


def test_normalize_angle_matches_reference_formula():
    for a in [-10.0, -3.2, -np.pi, -1.0, 0.0, 0.5, np.pi, 3.5, 7.0, 100.0]:
        a32 = np.float32(a)
        r = np.fmod(np.float32(a32 + np.float32(np.pi)), np.float32(2 * np.pi))
        ref = r + np.float32(np.pi) if r <= 0 else r - np.float32(np.pi)
        assert np.float32(oracle.normalize_angle(a32)) == np.float32(ref)


def test_smoothing_known_answer():
    # controller_generic_tests.cu:214-237: u[0] kept; with T = 2, u(:,1) = 61/35
    u = np.array([[1.0], [2.0]], dtype=np.float32)
    out = oracle.smooth(u[:1])
    assert out[0, 0] == 1.0
    out = oracle.smooth(u)
    assert out[0, 0] == 1.0
    assert abs(out[1, 0] - 61.0 / 35.0) <= 4 * ulp(61.0 / 35.0)


def test_slide_known_answer():
    # controller_generic_tests.cu:239-282 (slide_control_scale = 0, zero control = 0)
    T, Cd = 100, 3
    u = np.repeat(np.arange(T, dtype=np.float32)[:, None], Cd, axis=1)
    z = np.zeros(Cd, np.float32)
    u1 = oracle.slide(u, 1, z, z)
    for i in range(T):
        expect = 0.0 if i + 1 > T - 1 else min(i + 1, T - 1)
        assert (u1[i] == expect).all()
    u2 = oracle.slide(u1, 10, z, z)
    for i in range(T):
        expect = 0.0 if i + 10 > T - 2 else min(i + 11, T - 1)
        assert (u2[i] == expect).all()


def test_cartpole_equilibrium():
    # cartpole_dynamics_tests.cu:24-45
    dyn = A.CartpoleParams(1.0, 1.0, 1.0, 9.81)
    cost = A.CartpoleCostParams(10, 1, 100, 1, 0)
    for fp64 in (True, False):
        xd = oracle.dynamics_deriv(A.MODEL_CARTPOLE, dyn, cost, np.zeros(4), np.zeros(1), fp64=fp64)
        assert np.abs(xd).max() < 1e-4


def test_normexp_known_answers(golden):
    k = golden["kats"]
    _, b, _ = oracle.weights(k["baseline_costs"], lambda_inv=1.0)
    assert np.float32(b) == k["baseline_known"][0]
    w, b, n = oracle.weights(k["expnorm_costs"], lambda_inv=np.float32(0.3))
    known = k["expnorm_known"]
    assert np.all(np.abs(w - known) <= 4 * ulp(known))
    assert abs(n - float(np.sum(known.astype(np.float64)))) < 1e-9 * n


def test_weighted_reduction_known_answer(golden):
    k = golden["kats"]
    out, absout = oracle.weighted_mean(k["wr_weights"], k["wr_normalizer"][0], k["wr_controls"], 1024, 100, 4)
    assert np.allclose(out, k["wr_known"], rtol=1e-12, atol=0)


def colored_case(golden, case):
    g = golden["colored"]
    T = int(g[f"c{case}_T"])
    zr, zi = g[f"c{case}_zr"], g[f"c{case}_zi"]
    spec = np.stack([zr, zi], axis=-1)  # [batch][F][2]
    return T, float(g[f"c{case}_beta"]), float(g[f"c{case}_fmin"]), spec, g[f"c{case}_y"]


@pytest.mark.parametrize("case", range(6))
def test_colored_noise_matches_reference_script(golden, case):
    T, beta, fmin, spec, y = colored_case(golden, case)
    batch = spec.shape[0]
    eps = oracle.colored_noise(spec, batch, T, 1, [beta], fmin=fmin, decay=0.0, offset_t=0)
    ref = y[:, :T]
    err = np.abs(eps.reshape(batch, T) - ref)
    assert err.max() <= 2e-5 * max(1.0, np.abs(ref).max()), err.max()


def test_colored_scales_follow_fftfreq_cutoff():
    # colored_noise.cu:294-333: frequencies below max(fmin, 1/N) take the cutoff's scale
    s, sigma = oracle.colored_scales(4, 1, [2.0], fmin=0.0)
    f = np.arange(5) / 8.0
    f[0] = f[1]
    ref = f ** -1.0
    assert np.allclose(s[:, 0], ref, rtol=1e-6)
    w = ref[1:].copy()
    w[-1] *= 0.5
    assert math.isclose(sigma[0], 2 * np.sqrt(np.sum(w ** 2)) / 8, rel_tol=1e-6)


@pytest.mark.parametrize("gamma,r", [(5.0, 2.0), (20.0, 1.5), (2.5, 3.0)])
def test_tsallis_transform_restatement(gamma, r):
    """The oracle's TsallisTransform (mppi_common.cu:1004-1021) against a NumPy restatement of the same float
    arithmetic (1 - d / gamma formed in double, narrowed to float before the log): libm and NumPy round log / exp
    differently in the last place, and the exponent |log(1 - d / gamma)| / (r - 1) scales that, so the bound is a few
    ulps times that exponent; exactly 1 at the baseline, exactly 0 from d >= gamma on, non-increasing in the cost."""
    rng = np.random.default_rng(int(gamma * 10 + r))
    c = (100.0 + rng.exponential(gamma / 2, 4096)).astype(np.float32)
    b = np.float32(c.min())
    w = oracle.tsallis(c, gamma, r, b)
    d = (c - b).astype(np.float32)
    q = (d / np.float32(gamma)).astype(np.float32)
    arg = (1.0 - q.astype(np.float64)).astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        ref = np.where(d < np.float32(gamma),
                       np.exp(np.log(arg) / np.float32(np.float32(r) - np.float32(1.0))), 0.0).astype(np.float32)
    expo = np.abs(np.log(np.maximum(arg, np.float32(1e-30)).astype(np.float64))) / (r - 1.0)
    tol = 4.0 * 2.0 ** -23 * (1.0 + expo) * ref + 1e-30
    assert np.all(np.abs(w.astype(np.float64) - ref) <= tol)
    assert w[np.argmin(c)] == 1.0
    assert np.all(w[d >= np.float32(gamma)] == 0.0) and np.any(d >= np.float32(gamma))
    order = np.argsort(c, kind="stable")
    assert np.all(np.diff(w[order]) <= 0.0)


@pytest.mark.parametrize("case", range(4))
def test_tsallis_matches_reference_function(golden, case):
    """orc_tsallis bit for bit against the reference's own TsallisTransform (mppi_common.cu:1004-1021), compiled for
    the host from the reference checkout and run on the fixture's costs (tests/golden/make_golden.py)."""
    g = golden["tsallis"]
    w = oracle.tsallis(g[f"t{case}_costs"], float(g[f"t{case}_gamma"]), float(g[f"t{case}_r"]),
                       float(g[f"t{case}_baseline"]))
    assert np.array_equal(w.view(np.uint32), g[f"t{case}_weights"].view(np.uint32))


def test_cartpole_trig_choice_moves_costs_below_parity_tolerance():
    """The reference's host twin evaluates the cart-pole with libm sinf / cosf (cartpole_dynamics.cu:48-53), its
    device code with the __sinf / __cosf intrinsics after normalizeAngle (:87-105); the engine and the oracle use
    the engine's own sincos_f.  On the benchmark cart-pole rollout (K = 2048, T = 100, +-5 N clamp) the per-sample
    costs of the two float forms differ by at most 1e-5 relative (measured: median <= 1e-7, max ~1.3e-6) and both
    are equally close to the FP64 rollout."""
    K, T = 2048, 100
    rng = np.random.default_rng(0)
    dyn, cost = A.CartpoleParams(1, 1, 1, 9.81), A.CartpoleCostParams(10, 1, 100, 1, 0)
    sp, cc = A.default_sampling_params(native=False), A.default_constraints(native=False)
    cc.lower[0], cc.upper[0] = -5.0, 5.0
    for _ in range(3):
        x0 = np.array([rng.uniform(-0.1, 0.1), rng.uniform(-0.1, 0.1), rng.uniform(-np.pi, np.pi),
                       rng.uniform(-0.1, 0.1)], np.float32)
        u = np.clip(rng.standard_normal(K * T).astype(np.float32), -5, 5)
        own, _, _ = oracle.rollout(A.MODEL_CARTPOLE, dyn, cost, x0, u, u[:T], sp, cc, 1.0, 0.0, K, T, 0.02)
        with oracle.libm_trig():
            libm, _, _ = oracle.rollout(A.MODEL_CARTPOLE, dyn, cost, x0, u, u[:T], sp, cc, 1.0, 0.0, K, T, 0.02)
        c64, _, _ = oracle.rollout(A.MODEL_CARTPOLE, dyn, cost, x0, u, u[:T], sp, cc, 1.0, 0.0, K, T, 0.02,
                                   fp64=True)
        rel = np.abs(own - libm) / np.abs(libm)
        assert np.median(rel) <= 1e-6 and rel.max() <= 1e-5, (np.median(rel), rel.max())
        e_own, e_libm = np.abs(own - c64) / np.abs(c64), np.abs(libm - c64) / np.abs(c64)
        assert np.median(e_own) <= 2 * np.median(e_libm) + 1e-8 and e_own.max() <= 1e-5
    assert oracle.lib().orc_get_trig_mode() == 0
