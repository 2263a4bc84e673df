"""Kernel-level parity of the CUDA engine against the oracle, mirroring the reference's kernel tests
(tests/mppi_core/normexp_kernel_tests.cu, weightedreduction_kernel_tests.cu, rollout_kernel_tests.cu,
tests/sampling_distributions/gaussian_noise_tests.cu).  Every call goes through the C ABI."""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from mppi_generic_vendor_gb300 import _abi as A
from tests._gpu import dev, empty, host, ptr, stream

pytestmark = pytest.mark.gpu


def ulp(x):
    return np.spacing(np.abs(np.asarray(x, dtype=np.float32))).astype(np.float64)


def test_philox_raw_known_answers():
    for ctr, key, exp in [([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
                          ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
                          ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
                           [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1])]:
        out = empty(4, "int32")
        A.call("mppi_kernel_philox_raw", ptr(out), 1, (C.c_uint32 * 4)(*ctr), (C.c_uint32 * 2)(*key), stream())
        assert [int(v) & 0xFFFFFFFF for v in host(out)] == exp
    # a run of counters against the oracle's integer restatement
    out = empty(4 * 1000, "int32")
    A.call("mppi_kernel_philox_raw", ptr(out), 1000, (C.c_uint32 * 4)(5, 6, 7, 8), (C.c_uint32 * 2)(9, 10), stream())
    got = host(out).view(np.uint32).reshape(1000, 4)
    for i in (0, 1, 517, 999):
        assert list(got[i]) == oracle.philox4x32_10([5 + i, 6, 7, 8], [9, 10])


def test_sincos_bit_identical_to_oracle():
    rng = np.random.default_rng(1)
    x = np.concatenate([np.linspace(-np.pi, np.pi, 100001), rng.uniform(-1e3, 1e3, 100000)]).astype(np.float32)
    xs, s, c = dev(x), empty(x.size), empty(x.size)
    A.call("mppi_kernel_sincos", ptr(xs), ptr(s), ptr(c), x.size, stream())
    so, co = oracle.sincosf(x)
    assert np.array_equal(host(s).view(np.uint32), so.view(np.uint32))
    assert np.array_equal(host(c).view(np.uint32), co.view(np.uint32))


def sigma_bins(z):
    out = []
    for j in range(3):
        rule = 0.5 * (math.erf((j + 1) / math.sqrt(2.0)) - math.erf(-(j + 1) / math.sqrt(2.0)))
        frac = float(np.mean(np.abs(z) < j + 1))
        out.append(abs(frac - rule) / rule)
    return out


def test_philox_normals_are_gaussian():
    # gaussian_noise_tests.cu:114-179: 1/2/3-sigma bin fractions within 1e-3 relative
    n = 1 << 24
    out = empty(n)
    A.call("mppi_kernel_philox_normal", ptr(out), n, 42, 0, stream())
    z = host(out).astype(np.float64)
    assert abs(z.mean()) < 2e-3 and abs(z.std() - 1.0) < 2e-3
    assert max(sigma_bins(z)) < 1e-3


def test_weight_transform_known_answers(golden):
    k = golden["kats"]
    # baseline over 4196 N(100, 2) costs (normexp_kernel_tests.cu:45-60)
    c = dev(k["baseline_costs"])
    o = empty(2)
    A.call("mppi_kernel_weight_transform", ptr(c), ptr(o), 1.0, c.numel(), 1, stream())
    assert host(o)[0] == k["baseline_known"][0]
    # descending sequence, min = 1 (normexp_kernel_tests.cu:102-124)
    c = dev(np.arange(6048, 0, -1, dtype=np.float32))
    A.call("mppi_kernel_weight_transform", ptr(c), ptr(o), 1.0, 6048, 1, stream())
    assert host(o)[0] == 1.0
    # expf(-0.3 (c - min)) over 555 costs (normexp_kernel_tests.cu:126-150), ASSERT_FLOAT_EQ = 4 ulp
    c = dev(k["expnorm_costs"])
    A.call("mppi_kernel_weight_transform", ptr(c), ptr(o), 0.3, 555, 1, stream())
    w = host(c)
    assert np.all(np.abs(w - k["expnorm_known"]) <= 4 * ulp(k["expnorm_known"]))
    assert abs(host(o)[1] - k["expnorm_known"].astype(np.float64).sum()) <= 4 * ulp(host(o)[1])


def test_weight_transform_matches_host_method():
    # normexp_kernel_tests.cu:180-256 (host baseline/normaliser vs device transform), several systems per launch
    rng = np.random.default_rng(7)
    lam = np.float32(0.3)
    K, nsys = 10000, 5
    costs = rng.normal(100.0, 2.0, size=(nsys, K)).astype(np.float32)
    c = dev(costs.reshape(-1))
    o = empty(2 * nsys)
    linv = np.float32(1.0) / lam
    A.call("mppi_kernel_weight_transform", ptr(c), ptr(o), float(linv), K, nsys, stream())
    w_gpu = host(c).reshape(nsys, K)
    bn = host(o).reshape(nsys, 2)
    for s in range(nsys):
        w, b, n = oracle.weights(costs[s], lambda_inv=linv)
        assert bn[s, 0] == b
        assert np.all(np.abs(w_gpu[s] - w) <= 4 * ulp(w))
        assert abs(bn[s, 1] - n) <= 1e-6 * n


def test_weighted_reduction_known_answer(golden):
    # weightedreduction_kernel_tests.cu:135-172 recipe (K=1024, T=100, C=4); tolerance 1e-5 relative to the sum of
    # absolute terms, the conditioning of a weighted sum
    k = golden["kats"]
    w, u = dev(k["wr_weights"]), dev(k["wr_controls"])
    bn = dev(np.array([0.0, k["wr_normalizer"][0]], dtype=np.float32))
    out = empty(400)
    A.call("mppi_kernel_weighted_reduction", ptr(w), ptr(u), ptr(out), ptr(bn), 0, 100, 1024, 4, stream())
    got = host(out)
    ref, absref = oracle.weighted_mean(k["wr_weights"], k["wr_normalizer"][0], k["wr_controls"], 1024, 100, 4)
    assert np.allclose(ref, k["wr_known"], rtol=1e-12)
    assert np.all(np.abs(got - ref) <= 1e-5 * absref)


def test_reduction_sum_known_answer(golden):
    # the normaliser known answer of normexp_kernel_tests.cu:62-79 (sum in double) through the reduction kernel
    k = golden["kats"]
    w = dev(k["normalizer_costs"])
    u = dev(np.ones(1024, np.float32))
    bn = dev(np.array([0.0, 1.0], dtype=np.float32))
    out = empty(1)
    A.call("mppi_kernel_weighted_reduction", ptr(w), ptr(u), ptr(out), ptr(bn), 0, 1, 1024, 1, stream())
    assert abs(host(out)[0] - k["normalizer_known"][0]) <= 4 * ulp(k["normalizer_known"][0])


@pytest.mark.parametrize("Cd,stride,decay,pure", [(1, 1, 1.0, 0.01), (2, 0, 0.9, 0.05), (2, 5, 1.0, 0.0),
                                                  (1, 3, 0.5, 1.0)])
def test_gaussian_controls_bit_identical(Cd, stride, decay, pure):
    # setGaussianControls (gaussian.cu:17-277) + enforceConstraints (dynamics.cu:107-126)
    rng = np.random.default_rng(11)
    K, T = 1000, 37
    eps = rng.standard_normal(K * T * Cd).astype(np.float32)
    mean = rng.uniform(-1, 1, T * Cd).astype(np.float32)
    std = np.array([1.3, 0.4][:Cd], dtype=np.float32)
    cc = A.default_constraints()
    for i in range(Cd):
        cc.lower[i], cc.upper[i], cc.deadband[i] = -1.5, 1.2, 0.05 * i
    s, mean_d = dev(eps), dev(mean)  # keep the device buffers alive until the kernel has run
    A.call("mppi_kernel_gaussian_controls", ptr(s), ptr(mean_d), std.ctypes.data_as(C.POINTER(C.c_float)),
           C.byref(cc), K, T, Cd, stride, decay, pure, stream())
    ref = oracle.gaussian_rewrite(eps, mean, std, K, T, Cd, stride, decay, pure)
    ref = oracle.enforce_constraints(ref, Cd, cc)
    assert np.array_equal(host(s).view(np.uint32), ref.view(np.uint32))


def _cartpole():
    return A.CartpoleParams(1.0, 1.0, 1.0, 9.81), A.CartpoleCostParams(10.0, 1.0, 100.0, 1.0, 0.5)


def _di():
    p = A.DIObstacleCostParams()
    p.goal[:] = [3.0, -2.0, 0.0, 0.0]
    p.coeff[:] = [1.0, 1.0, 0.1, 0.1]
    p.terminal_coeff = 10.0
    p.num_obstacles = 8
    rng = np.random.default_rng(5)
    for j in range(8):
        p.obstacle_x[j], p.obstacle_y[j] = rng.uniform(-5, 5, 2)
        p.obstacle_radius[j] = rng.uniform(0.3, 1.0)
    p.obstacle_cost = 1000.0
    return A.DoubleIntegratorParams(0.0), p


@pytest.mark.parametrize("model,K,T,Cd,cc_coeff", [(A.MODEL_CARTPOLE, 2048, 100, 1, 0.0),
                                                    (A.MODEL_CARTPOLE, 300, 37, 1, 0.5),
                                                    (A.MODEL_DOUBLE_INTEGRATOR, 1024, 64, 2, 0.0),
                                                    (A.MODEL_DOUBLE_INTEGRATOR, 77, 30, 2, 0.2)])
def test_rollout_costs_bit_identical(model, K, T, Cd, cc_coeff):
    # rollout_kernel_tests.cu:200-261 compares GPU and CPU rollouts at 1e-4; the engine matches the float oracle
    # bit for bit and is compared with the FP64 rollout for accuracy
    dyn, cost = _cartpole() if model == A.MODEL_CARTPOLE else _di()
    rng = np.random.default_rng(K + T)
    x0 = (np.array([0.1, 0.0, 2.5, 0.0]) if model == A.MODEL_CARTPOLE else np.array([-4.0, 4.0, 0.5, 0.0]))
    x0 = x0.astype(np.float32)
    u = np.clip(rng.normal(0, 1.5, K * T * Cd), -5, 5).astype(np.float32)
    mean = rng.uniform(-0.5, 0.5, T * Cd).astype(np.float32)
    sp = A.default_sampling_params()
    for i in range(Cd):
        sp.control_cost_coeff[i] = cc_coeff
    cc = A.default_constraints()
    costs = empty(K)
    x0_d, u_d, mean_d = dev(x0), dev(u), dev(mean)  # keep the device buffers alive until the kernel has run
    A.call("mppi_kernel_rollout", model, C.byref(dyn), C.sizeof(dyn), C.byref(cost), C.sizeof(cost), C.byref(sp),
           ptr(x0_d), ptr(u_d), ptr(mean_d), ptr(costs), K, T, 0.02, 1.0, 0.0, stream())
    got = host(costs)
    ref, _, _ = oracle.rollout(model, dyn, cost, x0, u, mean, sp, cc, 1.0, 0.0, K, T, 0.02)
    assert np.array_equal(got.view(np.uint32), ref.astype(np.float32).view(np.uint32))
    ref64, _, _ = oracle.rollout(model, dyn, cost, x0, u, mean, sp, cc, 1.0, 0.0, K, T, 0.02, fp64=True)
    rel = np.abs(got - ref64) / np.abs(ref64)
    assert np.median(rel) < 1e-5
