"""Learned surrogate: the GPU forward/backward kernels' gradients against the oracle's FP64 hand back-propagation
(itself checked against finite differences in test_oracle_surrogate.py), training convergence and determinism."""
import ctypes as C

import numpy as np
import pytest

import oracle
from mppi_generic_vendor_gb300 import _abi as A
from mppi_generic_vendor_gb300.surrogate import Surrogate

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("batch", [64, 200, 1000])
def test_gradient_matches_oracle(batch):
    s = Surrogate(num_transitions=4096, seed=3)
    rng = np.random.default_rng(batch)
    X = rng.normal(0, 1, (batch, 9)).astype(np.float32)
    Y = rng.normal(0, 1, (batch, 5)).astype(np.float32)
    loss, g = s.gradient(X, Y)
    p = s.params()[:A.MLP_WEIGHTS].astype(np.float64)
    ref_loss, ref = oracle.mlp_loss_grad(p, X, Y)
    assert abs(loss - ref_loss) <= 1e-5 * ref_loss
    # FP32 kernels vs FP64 reference: 1e-4 of the gradient's scale per parameter group
    for lo, hi in [(0, 576), (576, 640), (640, 4736), (4736, 4800), (4800, 5120), (5120, 5125)]:
        scale = np.abs(ref[lo:hi]).max()
        assert np.abs(g[lo:hi] - ref[lo:hi]).max() <= 1e-4 * scale + 1e-9, (lo, hi)
    s.close()


@pytest.mark.parametrize("fmt,precision", [("fp8", 1), ("bf16", 0)])
def test_quantisation_aware_gradient_matches_oracle(fmt, precision):
    """Quantisation-aware training: the training kernels' gradient in a 16-bit or FP8 weight format is the oracle's
    FP64 gradient of the network whose weights are the rounded ones the rollout holds (BF16 values, or E4M3 q times
    the per-layer power-of-two scale that mppi_mlp_quantize picks)."""
    s = Surrogate(num_transitions=4096, seed=3)
    s.set_weight_format(fmt)
    rng = np.random.default_rng(40 + precision)
    X = rng.normal(0, 1, (256, 9)).astype(np.float32)
    Y = rng.normal(0, 1, (256, 5)).astype(np.float32)
    loss, g = s.gradient(X, Y)
    p = s.params()
    q = np.empty(A.MLP_PARAMS, np.float32)
    sc = np.empty(3, np.float32)
    A.call("mppi_mlp_quantize", p.ctypes.data_as(C.POINTER(C.c_float)), precision,
           q.ctypes.data_as(C.POINTER(C.c_float)), sc.ctypes.data_as(C.POINTER(C.c_float)))
    w = q[:A.MLP_WEIGHTS].astype(np.float64)
    for l, (lo, hi) in enumerate([(0, 576), (640, 4736), (4800, 5120)]):
        w[lo:hi] *= sc[l]
        if precision == 0:  # BF16: the device rounds the FP32 weights itself
            u = p[lo:hi].astype(np.float32).view(np.uint32).astype(np.uint64)
            w[lo:hi] = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32).view(np.float32)
    assert not np.array_equal(w[:576], p[:576])  # the rounding is not the identity
    ref_loss, ref = oracle.mlp_loss_grad(w, X, Y)
    assert abs(loss - ref_loss) <= 1e-5 * ref_loss
    for lo, hi in [(0, 576), (576, 640), (640, 4736), (4736, 4800), (4800, 5120), (5120, 5125)]:
        scale = np.abs(ref[lo:hi]).max()
        assert np.abs(g[lo:hi] - ref[lo:hi]).max() <= 1e-4 * scale + 1e-9, (lo, hi)
    s.close()


def test_training_converges_and_is_deterministic():
    runs = []
    for _ in range(2):
        s = Surrogate(num_transitions=1 << 18, seed=11)
        s.generate()
        loss = s.train(steps=1500, batch=4096, lr=3e-3, lr_final=2e-4)
        runs.append((loss, s.params(), s.validate(1 << 15)))
        s.close()
    (l1, p1, r1), (l2, p2, r2) = runs
    assert np.array_equal(p1, p2) and np.array_equal(l1, l2)
    assert l1[-50:].mean() < 0.02 * l1[:10].mean(), (l1[:10].mean(), l1[-50:].mean())
    # a short run (1500 steps on 2^18 transitions) already predicts every derivative to within 15% of its spread
    out_std = p1[A.MLP_PARAMS - 5:]
    assert np.all(r1 < 0.15 * out_std), (r1, out_std)
