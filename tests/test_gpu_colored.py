"""Colored-noise sampler parity (ColoredNoiseDistributionImpl::generateSamples, colored_noise.cu:285-392).

Pinned three ways: against the reference's own NumPy generator (scripts/colored_noise.py) given the same spectrum
normals (golden fixture), against the oracle's FP64 direct transform inside a full batched computeControl, and
statistically with white (exponent 0) Philox noise as in colored_noise_tests.cu:98-200.  The engine evaluates the
inverse FFT in FP32, so noise values agree to ~1e-6; the tolerance below is 2e-5 of the noise scale.
"""
import math

import numpy as np
import pytest

import oracle
from mppi_generic_vendor_gb300 import (BatchedMPPIController, CartpoleDynamics, CartpoleSwingupCost,
                                       ColoredNoiseDistribution, DoubleIntegratorDynamics,
                                       DoubleIntegratorObstacleCost)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", range(6))
def test_colored_noise_matches_reference_script(golden, case):
    g = golden["colored"]
    T = int(g[f"c{case}_T"])
    beta, fmin = float(g[f"c{case}_beta"]), float(g[f"c{case}_fmin"])
    zr, zi, y = g[f"c{case}_zr"], g[f"c{case}_zi"], g[f"c{case}_y"]
    batch = zr.shape[0]
    F = T + 1
    # sample 0 of a controller is the nominal sequence itself, so the golden rows go to samples 1..batch
    spec = np.zeros((batch + 1, 1, F, 2), np.float32)
    spec[1:, 0, :, 0] = zr
    spec[1:, 0, :, 1] = zi
    sampler = ColoredNoiseDistribution(std_dev=(1.0,), exponents=(beta,), fmin=fmin, offset_decay_rate=0.0,
                                       pure_noise_trajectories_percentage=0.0)
    ctrl = BatchedMPPIController(CartpoleDynamics(), CartpoleSwingupCost(), sampler, [batch + 1], [T])
    ctrl.injectNoise(spec)
    ctrl.generateSamples(0, 0)
    eps = ctrl.control_samples().reshape(batch + 1, T)[1:]
    ref = y[:, :T]
    err = np.abs(eps - ref).max()
    assert err <= 2e-5 * max(1.0, np.abs(ref).max()), err
    ctrl.close()


@pytest.mark.parametrize("T,stride", [(32, 0), (32, 40), (64, 69), (64, 17), (128, 127), (128, 200), (50, 7)])
def test_colored_noise_offsets_match_oracle(T, stride):
    """Every offset branch of the transforms: x[stride] from the first or the second half of the length-2T sequence,
    odd and even offsets, the two-threads-per-row kernel (T = 32, 64, 128) and the direct transform (T = 50); two
    controls with different exponents, injected spectrum, against the oracle's FP64 transform."""
    K, C = 300, 2
    rng = np.random.default_rng(T + stride)
    spec = rng.standard_normal(K * C * (T + 1) * 2).astype(np.float32)
    sampler = ColoredNoiseDistribution(std_dev=(1.0, 1.0), exponents=(1.0, 0.5), offset_decay_rate=0.9,
                                       pure_noise_trajectories_percentage=0.0)
    ctrl = BatchedMPPIController(DoubleIntegratorDynamics(), [DoubleIntegratorObstacleCost()], sampler, [K], [T])
    ctrl.injectNoise(spec)
    ctrl.generateSamples(stride, 0)
    got = ctrl.control_samples().reshape(K, T, C)
    ref = oracle.colored_noise(spec, K, T, C, [1.0, 0.5], fmin=0.0, decay=0.9, offset_t=stride).reshape(K, T, C)
    err = np.abs(got[1:, stride:] - ref[1:, stride:]).max() if stride < T else 0.0
    assert err <= 2e-5 * max(1.0, np.abs(ref).max()), err
    assert np.all(got[:, :min(stride, T)] == 0.0)  # the nominal (zero) sequence before the offset
    ctrl.close()


def test_colored_batched_compute_control_parity():
    rng = np.random.default_rng(31)
    Ks, Ts = [512, 1024, 256, 2048], [32, 64, 128, 50]
    costs = []
    for _ in Ks:
        obs = [(rng.uniform(-5, 5), rng.uniform(-5, 5), rng.uniform(0.3, 1.0)) for _ in range(8)]
        costs.append(DoubleIntegratorObstacleCost(goal=(rng.uniform(-4, 4), rng.uniform(-4, 4), 0, 0),
                                                  coeff=(1, 1, 0.1, 0.1), terminal_coeff=10.0, obstacles=obs))
    dyn = DoubleIntegratorDynamics()
    dyn.setControlRanges([(-1.0, 1.0), (-1.0, 1.0)])
    sampler = ColoredNoiseDistribution(std_dev=(0.5, 0.5), exponents=(1.0, 1.0))
    ctrl = BatchedMPPIController(dyn, costs, sampler, Ks, Ts)
    specs = [rng.standard_normal(K * 2 * (T + 1) * 2).astype(np.float32) for K, T in zip(Ks, Ts)]
    x0 = [rng.uniform(-5, 5, 4).astype(np.float32) for _ in Ks]
    init = [rng.uniform(-0.3, 0.3, (T, 2)).astype(np.float32) for T in Ts]
    ctrl.setControlSeqs([u.T for u in init])
    ctrl.injectNoise(np.concatenate(specs))
    ctrl.computeControl(np.concatenate(x0), 1)
    got_costs = ctrl.sample_costs()
    got_u = ctrl.getControlSeqs()
    koff = np.concatenate([[0], np.cumsum(Ks)])
    for i, (K, T) in enumerate(zip(Ks, Ts)):
        eps = oracle.colored_noise(specs[i], K, T, 2, [1.0, 1.0], fmin=0.0, decay=0.97, offset_t=1)
        ref = oracle.compute_control(ctrl.model_id, ctrl._dyn_arr[i], ctrl._cost_arr[i], ctrl.getParams(),
                                     sampler.to_c(), ctrl.constraints_, K, T, 2, 4, x0[i], eps, init[i], stride=1)
        gc = got_costs[koff[i]:koff[i + 1]]
        rel = np.abs(gc - ref["costs"]) / np.abs(ref["costs"])
        assert rel.max() < 1e-4 and np.median(rel) < 1e-5, (i, rel.max())
        scale = max(1.0, float(np.abs(ref["samples"]).max()))
        assert np.abs(got_u[i].T - ref["control"]).max() <= 1e-4 * scale
    ctrl.close()


def test_white_colored_noise_is_gaussian():
    # colored_noise_tests.cu:98-140: exponent 0 gives white Gaussian noise (1/2/3-sigma bins)
    K, T = 16384, 128
    sampler = ColoredNoiseDistribution(std_dev=(1.0,), exponents=(0.0,), offset_decay_rate=0.0,
                                       pure_noise_trajectories_percentage=1.0)
    ctrl = BatchedMPPIController(CartpoleDynamics(), CartpoleSwingupCost(), sampler, [K], [T], seed=42)
    ctrl.generateSamples(0, 0)
    z = ctrl.control_samples().reshape(K, T)[1:].astype(np.float64).reshape(-1)
    assert abs(z.mean()) < 5e-3 and abs(z.std() - 1.0) < 5e-3
    for j in range(3):
        rule = 0.5 * (math.erf((j + 1) / math.sqrt(2.0)) - math.erf(-(j + 1) / math.sqrt(2.0)))
        frac = float(np.mean(np.abs(z) < j + 1))
        assert abs(frac - rule) / rule < 1.5e-3, (j, frac, rule)
    ctrl.close()


def test_pink_noise_spectrum_slope():
    # exponent 1: the periodogram of the generated noise falls as 1/f
    K, T = 4096, 128
    sampler = ColoredNoiseDistribution(std_dev=(1.0,), exponents=(1.0,), offset_decay_rate=0.0,
                                       pure_noise_trajectories_percentage=1.0)
    ctrl = BatchedMPPIController(CartpoleDynamics(), CartpoleSwingupCost(), sampler, [K], [T], seed=5)
    ctrl.generateSamples(0, 0)
    z = ctrl.control_samples().reshape(K, T)[1:].astype(np.float64)
    p = (np.abs(np.fft.rfft(z, axis=1)) ** 2).mean(axis=0)[2:T // 2]
    f = np.arange(2, T // 2)
    slope = np.polyfit(np.log(f), np.log(p), 1)[0]
    assert -1.3 < slope < -0.7, slope
    ctrl.close()
