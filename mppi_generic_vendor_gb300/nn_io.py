"""Network weight files of the learned dynamics: the reference's FNNHelper npz format and the engine's own.

The reference stores a feed-forward network as double arrays ``dynamics_W{i}`` (shape [out][in], row-major, output
index first) and ``dynamics_b{i}`` (length out) for layers i = 1, 2, ..., optionally under a key prefix
(FNNHelper::loadParams, include/mppi/utils/nn_helpers/fnn_helper.cu:64-127).  It has no input or output
normalisation: the network maps raw inputs to raw outputs.  The engine's parameter vector (MPPI_MLP_PARAMS floats)
is the same three layers followed by in_mean[9], in_std[9], out_mean[5], out_std[5]; a network read from the
reference's format gets the identity normalisation, and a network written to it has the normalisation folded into
the first and last layers.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_OUT = 9, 64, 5
W1, B1 = 0, N_HID * N_IN
W2, B2 = B1 + N_HID, B1 + N_HID + N_HID * N_HID
W3 = B2 + N_HID
B3 = W3 + N_OUT * N_HID
IN_MEAN = B3 + N_OUT
IN_STD = IN_MEAN + N_IN
OUT_MEAN = IN_STD + N_IN
OUT_STD = OUT_MEAN + N_OUT
NUM_PARAMS = OUT_STD + N_OUT  # 5153 = MPPI_MLP_PARAMS
LAYERS = [(N_IN, N_HID, W1, B1), (N_HID, N_HID, W2, B2), (N_HID, N_OUT, W3, B3)]


def _key(prefix: str, name: str, i: int) -> str:
    if prefix and not prefix.endswith("/"):
        prefix += "/"
    return f"{prefix}dynamics_{name}{i}"


def is_reference_format(d, prefix: str = "") -> bool:
    return _key(prefix, "W", 1) in d and _key(prefix, "b", 1) in d


def from_reference(d, prefix: str = "") -> np.ndarray:
    """Engine parameter vector from a mapping holding the reference's ``dynamics_W{i}`` / ``dynamics_b{i}`` arrays
    (the layer sizes follow from the array sizes, as FNNHelper::loadParams derives them; they must be 9-64-64-5)."""
    p = np.zeros(NUM_PARAMS, np.float64)
    n_layers = 0
    while _key(prefix, "b", n_layers + 1) in d:
        n_layers += 1
    if n_layers != len(LAYERS):
        raise ValueError(f"the network has {n_layers} layers; the surrogate expects {len(LAYERS)} (9-64-64-5)")
    for i, (n_in, n_out, wo, bo) in enumerate(LAYERS, start=1):
        w = np.asarray(d[_key(prefix, "W", i)], np.float64).reshape(-1)
        b = np.asarray(d[_key(prefix, "b", i)], np.float64).reshape(-1)
        if b.size != n_out or w.size != n_in * n_out:
            raise ValueError(f"layer {i} is {w.size // max(b.size, 1)} -> {b.size}; the surrogate expects "
                             f"{n_in} -> {n_out}")
        p[wo:wo + n_in * n_out] = w
        p[bo:bo + n_out] = b
    if not np.all(np.isfinite(p)):
        raise ValueError("the network has non-finite parameters")
    p[IN_STD:IN_STD + N_IN] = 1.0
    p[OUT_STD:OUT_STD + N_OUT] = 1.0
    return p.astype(np.float32)


def to_reference(params, prefix: str = "") -> dict:
    """The reference's arrays for an engine parameter vector, normalisation folded in (in double precision):
    W1' = W1 diag(1 / in_std), b1' = b1 - W1' in_mean, W3' = diag(out_std) W3, b3' = out_std * b3 + out_mean."""
    p = np.asarray(params, np.float64).reshape(-1)
    if p.size != NUM_PARAMS:
        raise ValueError(f"surrogate parameter vector must hold {NUM_PARAMS} floats")
    m, s = p[IN_MEAN:IN_MEAN + N_IN], p[IN_STD:IN_STD + N_IN]
    om, os_ = p[OUT_MEAN:OUT_MEAN + N_OUT], p[OUT_STD:OUT_STD + N_OUT]
    out = {}
    for i, (n_in, n_out, wo, bo) in enumerate(LAYERS, start=1):
        w = p[wo:wo + n_in * n_out].reshape(n_out, n_in).copy()
        b = p[bo:bo + n_out].copy()
        if i == 1:
            w = w / s[None, :]
            b = b - w @ m
        if i == len(LAYERS):
            w = w * os_[:, None]
            b = b * os_ + om
        out[_key(prefix, "W", i)] = w
        out[_key(prefix, "b", i)] = b
    return out


def load(path, prefix: str = "") -> np.ndarray:
    """Parameter vector from an npz file in either format: the engine's checkpoint (``params``) or the reference's
    ``dynamics_W{i}`` / ``dynamics_b{i}`` arrays."""
    with np.load(path) as f:
        if "params" in f and not prefix:
            p = np.asarray(f["params"], np.float32).reshape(-1)
            if p.size != NUM_PARAMS:
                raise ValueError(f"surrogate parameter vector must hold {NUM_PARAMS} floats")
            return p
        if is_reference_format(f, prefix):
            return from_reference(f, prefix)
    raise ValueError(f"{path}: neither a surrogate checkpoint ('params') nor FNNHelper arrays "
                     f"('{_key(prefix, 'W', 1)}', ...)")


def save_reference(path, params, prefix: str = ""):
    """Write the network in the reference's npz format."""
    np.savez(path, **to_reference(params, prefix))
