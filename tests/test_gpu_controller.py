"""Controller-level parity of the engine against the oracle's computeControl, given the same injected standard-normal
noise (the parity definition of the port), plus the reference's controller behaviours: batching of uneven instances,
graph replay, receding horizon, NaN rejection, sampler statistics, free-energy statistics, autotune cache."""
import ctypes as C
import math

import numpy as np
import pytest

import _parity
import oracle
from mppi_generic_vendor_gb300 import (BatchedMPPIController, CartpoleDynamics, CartpoleSwingupCost,
                                       DoubleIntegratorDynamics, DoubleIntegratorObstacleCost, GaussianDistribution,
                                       MPPIError, VanillaMPPIController)
from mppi_generic_vendor_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def cartpole_controller(K=2048, T=100, iters=1, std=1.0, lam=1.0, seed=0):
    dyn = CartpoleDynamics(1.0, 1.0, 1.0)
    dyn.setControlRanges([(-5.0, 5.0)])
    cost = CartpoleSwingupCost(10.0, 1.0, 100.0, 1.0, 0.0)
    sampler = GaussianDistribution(std_dev=(std,))
    ctrl = VanillaMPPIController(dyn, cost, None, sampler, 0.02, iters, lam, 0.0, T, K, seed=seed)
    return ctrl, dyn, cost


def di_cost(rng):
    obs = [(rng.uniform(-5, 5), rng.uniform(-5, 5), rng.uniform(0.3, 1.0)) for _ in range(8)]
    goal = (rng.uniform(-4, 4), rng.uniform(-4, 4), 0.0, 0.0)
    return DoubleIntegratorObstacleCost(goal=goal, coeff=(1.0, 1.0, 0.1, 0.1), terminal_coeff=10.0, obstacles=obs,
                                        obstacle_cost=1000.0)


def oracle_solve(ctrl, i, x0, eps, control_tc, stride=1, dyn=None, cost=None):
    cp = ctrl.getParams()
    sp = ctrl.sampler_.to_c()
    K, T = int(ctrl.K[i]), int(ctrl.T[i])
    d = ctrl._dyn_arr[i] if dyn is None else dyn
    c = ctrl._cost_arr[i] if cost is None else cost
    return oracle.compute_control(ctrl.model_id, d, c, cp, sp, ctrl.constraints_, K, T, ctrl.Cdim, ctrl.S, x0, eps,
                                  control_tc, stride=stride)


def check_control(got_tc, ref, rtol=1e-5):
    """Element-wise: each updated control within rtol of the magnitude of the weighted terms it sums (_parity)."""
    T, Cdim = np.asarray(ref["control"]).shape
    return _parity.check_control(got_tc, ref, ref["weights"].size, T, Cdim, rtol=rtol)


def check_weights(w, ref_w, rtol=1e-5):
    """Every weight within rtol relative, with an absolute floor of the smallest normal float (weights that underflow
    to subnormals or zero carry no share of the update)."""
    assert np.all(np.abs(w - ref_w) <= rtol * ref_w + np.finfo(np.float32).tiny)


@pytest.mark.parametrize("iters", [1, 3])
def test_cartpole_compute_control_parity(iters):
    K, T = 2048, 100
    ctrl, dyn, cost = cartpole_controller(K, T, iters)
    rng = np.random.default_rng(2024)
    eps = rng.standard_normal(K * T).astype(np.float32)
    x0 = np.array([0.05, -0.02, rng.uniform(-np.pi, np.pi), 0.03], dtype=np.float32)
    u_init = rng.uniform(-1, 1, (T, 1)).astype(np.float32)
    ctrl.setControlSeqs([u_init.T])
    ctrl.injectNoise(eps)
    ctrl.computeControl(x0, 1)
    ref = oracle_solve(ctrl, 0, x0, eps, u_init)
    got_costs = ctrl.sample_costs()
    if iters == 1:
        # same inputs: per-sample costs and constrained samples are bit-identical, the baseline is exact
        assert np.array_equal(got_costs.view(np.uint32), ref["costs"].view(np.uint32))
        assert np.array_equal(ctrl.control_samples().view(np.uint32), ref["samples"].view(np.uint32))
        assert ctrl.getBaselineCost() == ref["baseline"]
        check_weights(ctrl.sample_weights(), ref["weights"])
        bn, n64 = ctrl.baseline_normalizer()
        assert abs(n64[0] - ref["normalizer"]) <= 1e-5 * ref["normalizer"]
        check_control(ctrl.getControlSeq().T, ref)
    else:
        # iterations 2 and 3 sample around an update that already differs by float rounding (the engine's FP32 sum
        # against the oracle's FP64 sum); the exponential weights amplify a cost difference dc by dc / lambda, so
        # the third update is held to 1e-3 of its term magnitude while the costs stay within 1e-5 relative
        assert np.median(np.abs(got_costs - ref["costs"]) / np.abs(ref["costs"])) < 1e-5
        check_control(ctrl.getControlSeq().T, ref, rtol=1e-3)
    st = ctrl.getTargetStateSeq().T
    assert np.allclose(st, ref["state_seq"], rtol=1e-4, atol=1e-4)
    ctrl.close()


def test_double_integrator_batched_parity():
    rng = np.random.default_rng(99)
    Ks = [512, 1024, 2048, 777, 4096, 100]
    Ts = [32, 64, 128, 50, 32, 17]
    costs = [di_cost(rng) for _ in Ks]
    dyn = DoubleIntegratorDynamics()
    dyn.setControlRanges([(-1.0, 1.0), (-1.0, 1.0)])
    ctrl = BatchedMPPIController(dyn, costs, GaussianDistribution(std_dev=(0.5, 0.5)), Ks, Ts, dt=0.02,
                                 max_iter=1, lambda_=1.0)
    eps = [rng.standard_normal(K * T * 2).astype(np.float32) for K, T in zip(Ks, Ts)]
    x0 = [rng.uniform(-5, 5, 4).astype(np.float32) for _ in Ks]
    init = [rng.uniform(-0.5, 0.5, (T, 2)).astype(np.float32) for T in Ts]
    ctrl.setControlSeqs([u.T for u in init])
    ctrl.injectNoise(np.concatenate(eps))
    ctrl.computeControl(np.concatenate(x0), 1)
    got_costs = ctrl.sample_costs()
    got_u = ctrl.getControlSeqs()
    bn, _ = ctrl.baseline_normalizer()
    koff = np.concatenate([[0], np.cumsum(Ks)])
    for i in range(len(Ks)):
        ref = oracle_solve(ctrl, i, x0[i], eps[i], init[i])
        gc = got_costs[koff[i]:koff[i + 1]]
        assert np.array_equal(gc.view(np.uint32), ref["costs"].view(np.uint32)), i
        assert bn[i, 0] == ref["baseline"]
        check_control(got_u[i].T, ref)
    ctrl.close()


def test_graph_replay_matches_stream_launches():
    K, T = 1024, 64
    outs = []
    for graph in (True, False):
        ctrl, _, _ = cartpole_controller(K, T, iters=2, seed=7)
        ctrl.setGraphMode(graph)
        x0 = np.array([0.0, 0.0, 0.3, 0.0], np.float32)
        for _ in range(3):
            ctrl.computeControl(x0, 1)
            ctrl.slideControlSequence(1)
        outs.append((ctrl.getControlSeq().copy(), ctrl.sample_costs().copy()))
        ctrl.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_philox_noise_changes_every_call_and_is_reproducible():
    a, _, _ = cartpole_controller(256, 32, seed=3)
    b, _, _ = cartpole_controller(256, 32, seed=3)
    x0 = np.array([0.0, 0.0, 1.0, 0.0], np.float32)
    a.computeControl(x0)
    s1 = a.control_samples().copy()
    a.computeControl(x0)
    s2 = a.control_samples().copy()
    b.computeControl(x0)
    assert not np.array_equal(s1, s2)
    assert np.array_equal(s1, b.control_samples())
    a.close()
    b.close()


def test_cartpole_swing_up_receding_horizon():
    # vanilla_mppi_test.cu:79-136 style integration test: swing the pole up (theta = pi) with receding horizon
    ctrl, dyn, _ = cartpole_controller(2048, 100, iters=1, std=1.0, lam=1.0, seed=1)
    p = dyn.getParams()
    x = np.array([0.0, 0.0, 0.0, 0.0], np.float64)

    def f(x, u):
        s, c = math.sin(x[2]), math.cos(x[2])
        mc, mp, l, g = p.cart_mass, p.pole_mass, p.pole_length, p.gravity
        xdd = (u + mp * s * (l * x[3] ** 2 + g * c)) / (mc + mp * s * s)
        tdd = (-u * c - mp * l * x[3] ** 2 * c * s - (mc + mp) * g * s) / (l * (mc + mp * s * s))
        return np.array([x[1], xdd, x[3], tdd])

    upright = 0
    for step in range(500):
        ctrl.computeControl(x.astype(np.float32), 1)
        u = float(ctrl.getControlSeq()[0, 0])
        x = x + 0.02 * f(x, u)
        ctrl.slideControlSequence(1)
        if 1.0 + math.cos(x[2]) < 0.05:
            upright += 1
    assert upright > 100, upright
    ctrl.close()


def test_nan_state_is_rejected_and_handle_survives():
    ctrl, _, _ = cartpole_controller(256, 32)
    with pytest.raises(MPPIError) as e:
        ctrl.computeControl(np.array([0.0, np.nan, 0.0, 0.0], np.float32))
    assert e.value.status == 3
    ctrl.computeControl(np.zeros(4, np.float32))
    assert np.isfinite(ctrl.getBaselineCost())
    with pytest.raises(MPPIError):
        ctrl.injectNoise(np.full(256 * 32, np.nan, np.float32))
    ctrl.close()


def bins_ok(z):
    for j in range(3):
        rule = 0.5 * (math.erf((j + 1) / math.sqrt(2.0)) - math.erf(-(j + 1) / math.sqrt(2.0)))
        frac = float(np.mean(np.abs(z) < j + 1))
        assert abs(frac - rule) / rule < 1e-3, (j, frac, rule)


@pytest.mark.parametrize("pure", [0.0, 1.0])
def test_generate_samples_are_gaussian(pure):
    # gaussian_noise_tests.cu:114-245 (CheckSamplesAreGaussian / CheckZeroMeanSamplesAreGaussian)
    K, T = 8192, 128
    dyn = DoubleIntegratorDynamics()
    rng = np.random.default_rng(0)
    ctrl = BatchedMPPIController(dyn, di_cost(rng), GaussianDistribution(std_dev=(2.3, 2.3),
                                                                          pure_noise_trajectories_percentage=pure),
                                 [K], [T], seed=42)
    mean = rng.uniform(-1, 1, (T, 2)).astype(np.float32)
    ctrl.setControlSeqs([mean.T])
    ctrl.generateSamples(0, 0)
    s = ctrl.control_samples().reshape(K, T, 2)
    m = 0.0 if pure == 1.0 else mean[None]
    z = ((s - m) / 2.3)[1:]  # sample 0 is the mean
    bins_ok(z.reshape(-1).astype(np.float64))
    ctrl.close()


def test_free_energy_statistics():
    K, T = 1024, 50
    ctrl, _, _ = cartpole_controller(K, T)
    ctrl.computeControl(np.array([0, 0, 2.0, 0], np.float32))
    w = ctrl.sample_weights().astype(np.float64)
    fe = ctrl.getFreeEnergyStatistics()
    lam = 1.0
    norm = w.sum() / K
    assert math.isclose(fe["freeEnergyMean"], -lam * math.log(norm) + ctrl.getBaselineCost(), rel_tol=1e-5)
    assert math.isclose(fe["normalizerPercent"], ctrl.getNormalizerCost() / K, rel_tol=1e-6)
    ctrl.close()


def test_autotune_cache_roundtrip(tmp_path):
    cache = tmp_path / "tune.json"
    a, _, _ = cartpole_controller(1024, 32)
    a.autotune(cache)
    cfg = a.launchConfig()
    assert cache.exists() and '"m1_i1_' in cache.read_text()
    b, _, _ = cartpole_controller(1024, 32)
    b.autotune(cache)
    assert b.launchConfig() == cfg
    # results do not depend on the launch shape
    x0 = np.array([0, 0, 1.0, 0], np.float32)
    rng = np.random.default_rng(4)
    eps = rng.standard_normal(1024 * 32).astype(np.float32)
    outs = []
    for ns, kc in [(32, 64), (256, 256)]:
        c, _, _ = cartpole_controller(1024, 32)
        c.setLaunchConfig(ns, kc)
        c.injectNoise(eps)
        c.computeControl(x0)
        outs.append((c.sample_costs(), c.getControlSeq()))
        c.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.allclose(outs[0][1], outs[1][1], rtol=0, atol=1e-6)
    a.close()
    b.close()


@pytest.mark.parametrize("lik", [False, True])
def test_split_rollout_bit_identical_to_fused(lik):
    """Rollout modes 1 (dynamics chain, then all (k, t) costs in parallel), 2 (four lanes per sample), 3 (the
    sampler kernel, then the staged rollout) and 4 (fused with noise warps) give the fused kernel's samples and costs
    bit for bit, with and without the likelihood-ratio term, over several iterations of Philox noise (T = 100 is not
    a multiple of the cooperative kernel's 16-step groups)."""
    outs = []
    for mode in (0, 1, 2, 3, 4):
        dyn = CartpoleDynamics(1.0, 1.0, 1.0)
        dyn.setControlRanges([(-5.0, 5.0)])
        sampler = GaussianDistribution(std_dev=(1.0,), control_cost_coeff=(1.0,) if lik else (0.0,))
        ctrl = VanillaMPPIController(dyn, CartpoleSwingupCost(10.0, 1.0, 100.0, 1.0, 0.0), None, sampler, 0.02, 3, 1.0,
                                     0.0, 100, 2048, seed=5)
        m, avail = ctrl.rolloutMode()
        assert m == 0 and avail == 31
        ctrl.setRolloutMode(mode)
        assert ctrl.rolloutMode()[0] == mode
        x0 = np.array([0.0, 0.0, 2.0, 0.0], np.float32)
        ctrl.computeControl(x0, 1)
        ctrl.computeControl(x0, 1)
        outs.append((ctrl.sample_costs(), ctrl.getControlSeq(), ctrl.control_samples(), ctrl.kernelsPerCompute()))
        ctrl.close()
    (c0, u0, s0, n0), (c1, u1, s1, n1), (c2, u2, s2, n2), (c3, u3, s3, n3), (c4, u4, s4, n4) = outs
    for c, u, smp in ((c1, u1, s1), (c2, u2, s2), (c3, u3, s3), (c4, u4, s4)):
        assert np.array_equal(s0, smp)
        assert np.array_equal(c0.view(np.uint32), c.view(np.uint32))
        assert np.array_equal(u0, u)
    # three iterations: modes 0 and 4 combine and (last iteration) smooth in the rollout, mode 2 launches the combine
    # kernel, which smooths in the last iteration, modes 1 and 3 one more kernel per iteration (the cost kernel, the
    # sampler)
    assert n0 == n4 == 3
    assert n2 == 2 * 3
    assert n1 == n3 == 3 * 3


def test_split_rollout_unavailable_for_colored_noise():
    rng = np.random.default_rng(0)
    ctrl = BatchedMPPIController(DoubleIntegratorDynamics(), [di_cost(rng)], A_colored(), [512], [32])
    assert ctrl.rolloutMode() == (0, 1)
    with pytest.raises(MPPIError):
        ctrl.setRolloutMode(1)
    ctrl.close()


def A_colored():
    from mppi_generic_vendor_gb300 import ColoredNoiseDistribution

    return ColoredNoiseDistribution(std_dev=(0.5, 0.5), exponents=(1.0, 1.0))


def test_cooperative_rollout_bit_identical_for_two_controls():
    """Modes 2, 3 and 4 with C = 2 (a quad holds two steps) on the kinematic bicycle: samples, costs and the update
    equal mode 0's bit for bit; the weights served after the tile reduction equal the oracle's within 1e-5."""
    from mppi_generic_vendor_gb300 import BicycleDynamics, CostmapCost
    from mppi_generic_vendor_gb300.workloads import gaussian_bump_costmap

    cmap = gaussian_bump_costmap(3, size=128)
    K, T = 3000, 50
    rng = np.random.default_rng(31)
    eps = rng.standard_normal(K * T * 2).astype(np.float32)
    init = rng.uniform(-0.3, 0.3, (T, 2)).astype(np.float32)
    x0 = np.array([6.0, 5.0, 0.4, 4.0], np.float32)
    outs = []
    for mode in (0, 2, 3, 4):
        cost = CostmapCost(map_coeff=1.0, speed_target=8.0, speed_coeff=1.0, steer_coeff=0.5, terminal_coeff=2.0,
                           costmap=cmap, resolution=0.1, origin=(0.0, 0.0))
        ctrl = VanillaMPPIController(BicycleDynamics(2.5), cost, None, GaussianDistribution(std_dev=(1.0, 0.3)), 0.02,
                                     1, 2.0, 0.0, T, K)
        ctrl.setRolloutMode(mode)
        ctrl.setControlSeq(init.T)
        ctrl.injectNoise(eps)
        ctrl.computeControl(x0, 1)
        outs.append((ctrl.sample_costs(), ctrl.getControlSeq(), ctrl.sample_weights(), ctrl.control_samples()))
        ref = oracle.compute_control(ctrl.model_id, ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.getParams(),
                                     ctrl.sampler_.to_c(), ctrl.constraints_, K, T, 2, 4, x0, eps, init,
                                     costmap=(cmap, 0.1, (0.0, 0.0)))
        check_weights(outs[-1][2], ref["weights"])
        check_control(outs[-1][1].T, ref)
        ctrl.close()
    c0, u0, w0, s0 = outs[0]
    for c2, u2, w2, s2 in outs[1:]:
        assert np.array_equal(s0, s2)
        assert np.array_equal(c0.view(np.uint32), c2.view(np.uint32))
        assert np.array_equal(u0, u2)
        assert np.array_equal(w0, w2)


def test_device_only_solves_match_compute_control():
    """enqueueSolve runs the same device work as computeControl, smoothing and constraints included: n device-only
    solves from the same start leave the nominal sequence computeControl produces after n calls."""
    outs = []
    for device_only in (False, True):
        ctrl, _, _ = cartpole_controller(1024, 64, iters=1, seed=11)
        x0 = np.array([0.0, 0.0, 0.5, 0.0], np.float32)
        ctrl.computeControl(x0, 1)  # uploads x0 and the nominal sequence
        if device_only:
            ctrl.enqueueSolve(1, 3)
            ctrl.synchronize()
        else:
            for _ in range(3):
                ctrl.computeControl(x0, 1)
        outs.append(ctrl.sample_costs())
        ctrl.close()
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))


def test_engines_with_different_horizons_coexist():
    """The fused rollout's shared-memory cap is a property of the kernel, shared by every engine: creating a second
    engine with a shorter horizon (smaller staging) must not break the first one's launches."""
    x0 = np.array([0.0, 0.0, 0.5, 0.0], np.float32)
    long_h, _, _ = cartpole_controller(1024, 200, seed=1)
    long_h.computeControl(x0, 1)
    short_h, _, _ = cartpole_controller(1024, 100, seed=2)
    short_h.computeControl(x0, 1)
    long_h.computeControl(x0, 1)  # 200 x 129 floats of staging per CTA, above the short engine's 100 x 129
    assert np.all(np.isfinite(long_h.getControlSeq()))
    long_h.close()
    short_h.close()


@pytest.mark.parametrize("lik", [False, True])
def test_sampled_trajectories_match_oracle(lik):
    """calculateSampledStateTrajectories (visualizeKernel's read-out): a random 1% of the samples plus the top five by
    weight are re-rolled on the GPU; their states equal the oracle's FP32 trajectories of the same constrained
    controls bit for bit, the top five are the five largest weights, and (step costs summed in step order) / T +
    terminal / T reproduces each sample's cost from the solve bit for bit (with and without the likelihood term)."""
    K, T = 1024, 60
    dyn = CartpoleDynamics(1.0, 1.0, 1.0)
    dyn.setControlRanges([(-5.0, 5.0)])
    sampler = GaussianDistribution(std_dev=(1.0,), control_cost_coeff=(1.0,) if lik else (0.0,))
    ctrl = VanillaMPPIController(dyn, CartpoleSwingupCost(10.0, 1.0, 100.0, 1.0, 0.0), None, sampler, 0.02, 1, 1.0,
                                 0.0, T, K, seed=3)
    x0 = np.array([0.1, 0.0, 2.5, 0.0], np.float32)
    init = np.random.default_rng(9).uniform(-1.0, 1.0, (T, 1)).astype(np.float32)
    ctrl.setControlSeq(init.T)
    ctrl.computeControl(x0, 1)
    ctrl.setPercentageSampledControlTrajectories(0.01)
    ctrl.setTopNSampledControlTrajectories(5)
    ctrl.calculateSampledStateTrajectories(seed=4)
    idx = ctrl.sampled_indices_
    assert idx.size == int(0.01 * K) + 5
    w = ctrl.sample_weights()
    assert np.array_equal(np.sort(w[idx[-5:]]), np.sort(w)[-5:])
    top = ctrl.getTopTransformedCosts()
    assert np.allclose(top, w[idx[-5:]] / ctrl.getNormalizerCost(), rtol=0, atol=0)
    samples = ctrl.control_samples().reshape(K, T, 1)
    _, _, traj = oracle.rollout(A.MODEL_CARTPOLE, ctrl._dyn_arr[0], ctrl._cost_arr[0], x0,
                                np.ascontiguousarray(samples[idx]), init, sampler.to_c(), ctrl.constraints_, 1.0, 0.0,
                                idx.size, T, 0.02, want_traj=True)
    got = np.stack([s.T for s in ctrl.getSampledOutputTrajectories()])  # [n][T][S]
    assert np.array_equal(got, traj.reshape(idx.size, T, 4).astype(np.float32))
    costs = ctrl.sample_costs()
    for j, k in enumerate(idx):
        running = np.float32(0.0)
        for c in ctrl.getSampledCostTrajectories()[j]:
            running = np.float32(running + c)
        cost = np.float32(running / np.float32(T)) + np.float32(ctrl.sampled_terminal_costs_[j] / np.float32(T))
        assert np.float32(cost).view(np.uint32) == costs[k].view(np.uint32), (j, k, cost, costs[k])
    ctrl.close()


def test_sampled_trajectories_reject_bad_indices():
    dyn = CartpoleDynamics(1.0, 1.0, 1.0)
    ctrl = VanillaMPPIController(dyn, CartpoleSwingupCost(), None, GaussianDistribution(std_dev=(1.0,)), 0.02, 1, 1.0,
                                 0.0, 20, 256)
    ctrl.computeControl(np.zeros(4, np.float32), 1)
    bad = np.array([0, 256], np.int32)
    out = np.empty(2 * 20 * 4, np.float32)
    with pytest.raises(MPPIError):
        A.call("mppi_get_sampled_trajectories", ctrl._h, 0, bad.ctypes.data_as(C.POINTER(C.c_int)), 2,
               out.ctypes.data_as(C.POINTER(C.c_float)), out.ctypes.data_as(C.POINTER(C.c_float)),
               out.ctypes.data_as(C.POINTER(C.c_float)), None)
    ctrl.close()


def test_bounded_wait_gives_up_and_handle_recovers():
    """Rollout mode 4's rollout warps poll a shared-memory progress word written by the CTA's noise warps, a bounded
    wait with nothing asynchronous in flight.  With the noise warps withholding their progress (a flag nothing sets)
    and the bound cut to 16 polls, every rollout warp gives up: the solve returns MPPI_ETIMEOUT and leaves no state
    behind, so the next solve with the default bound matches the oracle bit for bit."""
    K, T = 2048, 100
    ctrl, dyn, cost = cartpole_controller(K, T)
    if not (ctrl.rolloutMode()[1] >> 4) & 1:
        pytest.skip("rollout mode 4 is not available for this shape")
    ctrl.setRolloutMode(4)
    rng = np.random.default_rng(77)
    eps = rng.standard_normal(K * T).astype(np.float32)
    x0 = np.array([0.0, 0.0, 2.5, 0.0], np.float32)
    init = rng.uniform(-1, 1, (T, 1)).astype(np.float32)
    ctrl.setControlSeqs([init.T])
    ctrl.injectNoise(eps)
    A.call("mppi_set_wait_diagnostics", ctrl._h, 16, 1)
    with pytest.raises(MPPIError) as err:
        ctrl.computeControl(x0, 1)
    assert err.value.status == A.MPPI_ETIMEOUT
    A.call("mppi_set_wait_diagnostics", ctrl._h, 0, 0)
    ctrl.setControlSeqs([init.T])
    ctrl.computeControl(x0, 1)
    ref = oracle_solve(ctrl, 0, x0, eps, init)
    assert np.array_equal(ctrl.sample_costs().view(np.uint32), ref["costs"].view(np.uint32))
    check_control(ctrl.getControlSeq().T, ref)
    ctrl.close()
