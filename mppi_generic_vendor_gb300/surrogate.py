"""Learned dynamics surrogate for the dynamic bicycle (trained on the GPU by the engine's own kernels).

``Surrogate`` wraps the ``mppi_surrogate_*`` C ABI: transitions are drawn on the GPU from the analytic
``BicycleSlipDynamics``, a 9 -> 64 -> 64 -> 5 tanh MLP is trained with the engine's forward / backward / Adam kernels,
and the resulting parameter vector (weights + normalisation, MPPI_MLP_PARAMS floats) is what a controller with the
MLP model loads.  The reference only evaluates pre-trained networks (FNNHelper, utils/nn_helpers/fnn_helper.cu).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from .controller import BicycleSlipDynamics


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Surrogate:
    def __init__(self, dynamics: BicycleSlipDynamics | None = None, num_transitions: int = 1 << 20, seed: int = 7,
                 state_lower=None, state_upper=None, stream: int = 0):
        self.dynamics = dynamics or BicycleSlipDynamics()
        cfg = A.SurrogateConfig()
        A.lib().mppi_default_surrogate_config(C.byref(cfg))
        cfg.num_transitions = int(num_transitions)
        cfg.seed = int(seed)
        if state_lower is not None:
            cfg.state_lower[:] = [float(v) for v in state_lower]
        if state_upper is not None:
            cfg.state_upper[:] = [float(v) for v in state_upper]
        self.config = cfg
        h = C.c_void_p()
        p = self.dynamics.getParams()
        A.call("mppi_surrogate_create", C.byref(p), C.byref(cfg), C.c_void_p(stream or None), C.byref(h))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            A.lib().mppi_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def generate(self):
        A.call("mppi_surrogate_generate", self._h)

    WEIGHT_FORMATS = {"bf16": 0, "fp8": 1, "fp32": 2}

    def set_weight_format(self, fmt: str):
        """Quantisation-aware training: the forward and backward passes of later train() / gradient() calls use the
        weights rounded as the tensor cores will hold them ("bf16", or "fp8": E4M3 with the per-layer power-of-two
        scale) while Adam updates the FP32 master weights; "fp32" (the default) trains the weights as they are."""
        A.call("mppi_surrogate_set_weight_format", self._h, self.WEIGHT_FORMATS[fmt])

    def train(self, steps=3000, batch=8192, lr=3e-3, lr_final=1e-4) -> np.ndarray:
        loss = np.empty(steps, dtype=np.float32)
        A.call("mppi_surrogate_train", self._h, int(steps), int(batch), float(lr), float(lr_final), _fp(loss))
        return loss

    def gradient(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, 9)
        Y = np.ascontiguousarray(Y, dtype=np.float32).reshape(-1, 5)
        g = np.empty(A.MLP_WEIGHTS, dtype=np.float32)
        loss = C.c_float()
        A.call("mppi_surrogate_gradient", self._h, _fp(X), _fp(Y), X.shape[0], _fp(g), C.byref(loss))
        return loss.value, g

    def validate(self, n=1 << 16) -> np.ndarray:
        out = np.empty(5, dtype=np.float32)
        A.call("mppi_surrogate_validate", self._h, int(n), _fp(out))
        return out

    def params(self) -> np.ndarray:
        out = np.empty(A.MLP_PARAMS, dtype=np.float32)
        A.call("mppi_surrogate_get_params", self._h, _fp(out))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != A.MLP_PARAMS:
            raise ValueError(f"expected {A.MLP_PARAMS} parameters")
        A.call("mppi_surrogate_set_params", self._h, _fp(p))

    def save(self, path, format="engine"):
        """Checkpoint as an .npz file: ``format="engine"`` stores weights, normalisation and the generating
        configuration; ``format="reference"`` stores the reference's FNNHelper arrays (normalisation folded in)."""
        if format == "reference":
            from . import nn_io

            nn_io.save_reference(path, self.params())
            return
        if format != "engine":
            raise ValueError("format must be 'engine' or 'reference'")
        np.savez(path, params=self.params(), seed=np.uint64(self.config.seed),
                 state_lower=np.array(self.config.state_lower[:], np.float32),
                 state_upper=np.array(self.config.state_upper[:], np.float32))

    def load(self, path, prefix=""):
        from . import nn_io

        self.set_params(nn_io.load(path, prefix))
