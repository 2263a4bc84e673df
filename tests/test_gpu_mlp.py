"""Surrogate MLP on the tensor cores (tcgen05, BF16 operands, FP32 accumulation in TMEM).

* ``mppi_kernel_mlp_forward`` against a NumPy emulation of the BF16 pipeline (operands rounded to BF16 as the kernel
  stores them, FP64 dot products, exact tanh) and against the oracle's FP64 forward on the FP32 parameters;
* the MLP bicycle controller against the oracle's FP32 MLP rollout on the same injected noise, and the drift of the
  surrogate rollout from the FP64 analytic rollout it was trained to imitate.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from _gpu import dev, empty, host, ptr, stream
from mppi_generic_vendor_gb300 import (BicycleSlipDynamics, BicycleSlipMLPDynamics, CostmapCost, GaussianDistribution,
                                       VanillaMPPIController)
from mppi_generic_vendor_gb300 import _abi as A
from mppi_generic_vendor_gb300.surrogate import Surrogate
from mppi_generic_vendor_gb300.workloads import gaussian_bump_costmap

pytestmark = pytest.mark.gpu

W1, B1, W2, B2, W3, B3 = 0, 576, 640, 4736, 4800, 5120
IN_MEAN, IN_STD, OUT_MEAN, OUT_STD = 5125, 5134, 5143, 5148


def bf16(a):
    """Round float32 to the nearest BF16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def emulate_bf16(p, X):
    """The kernel's arithmetic with exact dot products and tanh: BF16 weights and activations, FP32 bias/epilogue."""
    p = np.asarray(p, np.float32)
    xin = ((X.astype(np.float32) - p[IN_MEAN:IN_STD]) / p[IN_STD:OUT_MEAN]).astype(np.float32)
    a0 = bf16(xin).astype(np.float64)
    w1 = bf16(p[W1:B1]).reshape(64, 9).astype(np.float64)
    w2 = bf16(p[W2:B2]).reshape(64, 64).astype(np.float64)
    w3 = bf16(p[W3:B3]).reshape(5, 64).astype(np.float64)
    h1 = bf16(np.tanh((a0 @ w1.T).astype(np.float32) + p[B1:W2])).astype(np.float64)
    h2 = bf16(np.tanh((h1 @ w2.T).astype(np.float32) + p[B2:W3])).astype(np.float64)
    y = (h2 @ w3.T).astype(np.float32) + p[B3:IN_MEAN]
    return y * p[OUT_STD:] + p[OUT_MEAN:OUT_STD]


def random_params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(A.MLP_PARAMS, np.float32)
    p[W1:B1] = rng.normal(0, 1 / 3, 576)
    p[B1:W2] = rng.normal(0, 0.1, 64)
    p[W2:B2] = rng.normal(0, 1 / 8, 4096)
    p[B2:W3] = rng.normal(0, 0.1, 64)
    p[W3:B3] = rng.normal(0, 1 / 8, 320)
    p[B3:IN_MEAN] = rng.normal(0, 0.1, 5)
    p[IN_MEAN:IN_STD] = rng.uniform(-3, 3, 9)
    p[IN_STD:OUT_MEAN] = rng.uniform(0.5, 4, 9)
    p[OUT_MEAN:OUT_STD] = rng.uniform(-1, 1, 5)
    p[OUT_STD:] = rng.uniform(0.5, 5, 5)
    return p


def gpu_forward(p, X):
    Xd = dev(np.ascontiguousarray(X, np.float32))
    Yd = empty(X.shape[0] * 5)
    A.call("mppi_kernel_mlp_forward", p.ctypes.data_as(C.POINTER(C.c_float)), ptr(Xd), ptr(Yd), X.shape[0], stream())
    return host(Yd).reshape(-1, 5)


@pytest.mark.parametrize("batch", [1, 127, 128, 1000, 70001])
def test_forward_matches_bf16_emulation(batch):
    p = random_params(batch)
    rng = np.random.default_rng(100 + batch)
    X = (p[IN_MEAN:IN_STD] + p[IN_STD:OUT_MEAN] * rng.standard_normal((batch, 9))).astype(np.float32)
    got = gpu_forward(p, X)
    assert np.all(np.isfinite(got))
    emu = emulate_bf16(p, X)
    ref = oracle.mlp_forward(p[:A.MLP_WEIGHTS], ((X - p[IN_MEAN:IN_STD]) / p[IN_STD:OUT_MEAN]).astype(np.float32))
    ref = ref * p[OUT_STD:] + p[OUT_MEAN:OUT_STD]
    scale = p[OUT_STD:].astype(np.float64)
    # against the emulation only the accumulation order and tanh.approx differ: activations may land one BF16 step
    # apart, 2^-8 relative, which moves an output by well under 1% of its scale
    e_emu = np.abs(got - emu) / scale
    assert e_emu.max() < 1e-2, e_emu.max()
    # against FP64 on FP32 weights the BF16 rounding of weights and activations dominates: about 2^-9 relative per
    # operand, a few parts in a thousand of the output scale
    e64 = np.abs(got - ref) / scale
    assert np.sqrt((e64 ** 2).mean()) < 1e-2 and e64.max() < 5e-2, (np.sqrt((e64 ** 2).mean()), e64.max())


def test_forward_rejects_bad_parameters():
    p = random_params(1)
    p[IN_STD] = 0.0
    X = np.zeros((4, 9), np.float32)
    with pytest.raises(A.MPPIError):
        gpu_forward(p, X)


@pytest.fixture(scope="module")
def trained():
    s = Surrogate(num_transitions=1 << 18, seed=5)
    s.generate()
    s.train(steps=1500, batch=4096, lr=3e-3, lr_final=2e-4)
    p = s.params()
    rmse = s.validate(1 << 15)
    s.close()
    return p, rmse


def slip_cost(cmap):
    return CostmapCost(map_coeff=1.0, speed_target=8.0, speed_coeff=1.0, steer_coeff=0.5, terminal_coeff=2.0,
                       costmap=cmap, resolution=0.1, origin=(0.0, 0.0))


def test_mlp_controller_matches_oracle(trained):
    params, _ = trained
    K, T, lam, seed = 2048, 60, 2.0, 4
    cmap = gaussian_bump_costmap(seed, size=128)
    dyn = BicycleSlipMLPDynamics(params)
    ctrl = VanillaMPPIController(dyn, slip_cost(cmap), None, GaussianDistribution(std_dev=(0.5, 0.5)), 0.02, 1, lam,
                                 0.0, T, K)
    x0 = np.array([6.0, 5.0, 0.2, 6.0, 0.0, 0.0, 0.0], np.float32)
    rng = np.random.default_rng(seed)
    eps = rng.standard_normal(K * T * 2).astype(np.float32)
    init = rng.uniform(-0.2, 0.2, (T, 2)).astype(np.float32)
    ctrl.setControlSeq(init.T)
    ctrl.injectNoise(eps)
    ctrl.computeControl(x0, 1)
    got = ctrl.sample_costs()
    oracle.set_mlp(params)
    ref = oracle.compute_control(A.MODEL_BICYCLE_SLIP_MLP, ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.getParams(),
                                 ctrl.sampler_.to_c(), ctrl.constraints_, K, T, 2, 7, x0, eps, init,
                                 costmap=(cmap, 0.1, (0.0, 0.0)))
    # BF16 network inputs quantise the state to 2^-9 of its normalisation scale; over 60 steps that moves the
    # per-sample cost by a few parts in ten thousand
    rel = np.abs(got - ref["costs"]) / np.abs(ref["costs"])
    assert np.median(rel) < 2e-3 and rel.max() < 2e-2, (np.median(rel), rel.max())
    assert abs(ctrl.getBaselineCost() - ref["baseline"]) <= 2e-3 * abs(ref["baseline"])
    span = float(np.abs(ref["control"]).max())
    assert np.abs(ctrl.getControlSeq().T - ref["control"]).max() <= 5e-2 * span
    ctrl.close()


def test_surrogate_drift_from_fp64_analytic(trained):
    """The surrogate rollout (BF16 tensor cores) against the FP64 analytic model on the same constrained samples."""
    params, rmse = trained
    K, T, lam, seed = 2048, 60, 2.0, 6
    cmap = gaussian_bump_costmap(seed, size=128)
    sampler = GaussianDistribution(std_dev=(0.5, 0.5))
    ctrl = VanillaMPPIController(BicycleSlipMLPDynamics(params), slip_cost(cmap), None, sampler, 0.02, 1, lam, 0.0,
                                 T, K)
    x0 = np.array([20.0, 20.0, -0.4, 7.0, 0.0, 0.0, 0.0], np.float32)
    rng = np.random.default_rng(seed)
    eps = rng.standard_normal(K * T * 2).astype(np.float32)
    init = np.zeros((T, 2), np.float32)
    ctrl.setControlSeq(init.T)
    ctrl.injectNoise(eps)
    ctrl.computeControl(x0, 1)
    mlp_costs = ctrl.sample_costs()
    samples = ctrl.control_samples()
    analytic = BicycleSlipDynamics()
    r64, _, _ = oracle.rollout(A.MODEL_BICYCLE_SLIP, analytic.getParams(), ctrl._cost_arr[0], x0, samples, init,
                               sampler.to_c(), ctrl.constraints_, lam, 0.0, K, T, 0.02,
                               costmap=(cmap, 0.1, (0.0, 0.0)), fp64=True, state_dim=7)
    rel = np.abs(mlp_costs - r64) / np.abs(r64)
    # a 1500-step surrogate predicts per-step derivatives to within 15% of their spread; integrated over 1.2 s the
    # sample costs stay within a few percent of the exact model and rank the samples alike
    assert np.median(rel) < 5e-2, np.median(rel)
    order_mlp = np.argsort(mlp_costs)[: K // 100]
    order_64 = np.argsort(r64)[: K // 100]
    assert len(np.intersect1d(order_mlp, order_64)) >= K // 400
    ctrl.close()


def test_mlp_model_requires_weights():
    cmap = gaussian_bump_costmap(1, size=64)
    ctrl = VanillaMPPIController(BicycleSlipMLPDynamics(), slip_cost(cmap), None,
                                 GaussianDistribution(std_dev=(0.5, 0.5)), 0.02, 1, 2.0, 0.0, 20, 256)
    with pytest.raises(A.MPPIError):
        ctrl.computeControl(np.array([6.0, 5.0, 0.2, 6.0, 0.0, 0.0, 0.0], np.float32))
    ctrl.close()
