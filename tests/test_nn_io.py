"""Network files: the reference's FNNHelper npz arrays (dynamics_W{i} / dynamics_b{i}, fnn_helper.cu:64-127) and the
engine's own checkpoint load into the same surrogate parameter vector (no GPU)."""
import numpy as np
import pytest

from mppi_generic_vendor_gb300 import BicycleSlipMLPDynamics, nn_io


def _net(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(nn_io.NUM_PARAMS, np.float32)
    p[:nn_io.IN_MEAN] = rng.normal(0, 0.3, nn_io.IN_MEAN)
    p[nn_io.IN_MEAN:nn_io.IN_STD] = rng.normal(0, 2, 9)
    p[nn_io.IN_STD:nn_io.OUT_MEAN] = rng.uniform(0.5, 4, 9)
    p[nn_io.OUT_MEAN:nn_io.OUT_STD] = rng.normal(0, 1, 5)
    p[nn_io.OUT_STD:] = rng.uniform(0.5, 3, 5)
    return p


def _physical(p, X):
    """Raw outputs of the network with its normalisation, in FP64."""
    p = p.astype(np.float64)
    x = (X - p[nn_io.IN_MEAN:nn_io.IN_STD]) / p[nn_io.IN_STD:nn_io.OUT_MEAN]
    h = np.tanh(x @ p[:576].reshape(64, 9).T + p[576:640])
    h = np.tanh(h @ p[640:4736].reshape(64, 64).T + p[4736:4800])
    y = h @ p[4800:5120].reshape(5, 64).T + p[5120:5125]
    return y * p[nn_io.OUT_STD:] + p[nn_io.OUT_MEAN:nn_io.OUT_STD]


def test_reference_format_round_trip(tmp_path):
    p = _net(3)
    path = tmp_path / "net.npz"
    nn_io.save_reference(path, p)
    with np.load(path) as f:
        assert sorted(f.files) == ["dynamics_W1", "dynamics_W2", "dynamics_W3", "dynamics_b1", "dynamics_b2",
                                   "dynamics_b3"]
        assert f["dynamics_W1"].shape == (64, 9) and f["dynamics_W3"].shape == (5, 64)
        assert f["dynamics_W1"].dtype == np.float64
    dyn = BicycleSlipMLPDynamics()
    dyn.loadParams(path)
    q = dyn.mlp_params
    assert np.all(q[nn_io.IN_MEAN:nn_io.IN_STD] == 0) and np.all(q[nn_io.IN_STD:nn_io.OUT_MEAN] == 1)
    X = np.random.default_rng(4).normal(0, 3, (200, 9))
    a, b = _physical(p, X), _physical(q, X)
    assert np.abs(a - b).max() <= 1e-5 * max(1.0, np.abs(a).max())


def test_reference_format_with_prefix_and_checkpoint(tmp_path):
    p = _net(5)
    ref = nn_io.to_reference(p, prefix="model")
    np.savez(tmp_path / "pref.npz", **ref)
    assert set(ref) == {f"model/dynamics_{n}{i}" for n in "Wb" for i in (1, 2, 3)}
    q = nn_io.load(tmp_path / "pref.npz", prefix="model")
    X = np.random.default_rng(6).normal(0, 1, (50, 9))
    assert np.allclose(_physical(p, X), _physical(q, X), rtol=1e-5, atol=1e-5)
    np.savez(tmp_path / "own.npz", params=p)
    assert np.array_equal(nn_io.load(tmp_path / "own.npz"), p)


def test_reference_format_rejects_other_shapes(tmp_path):
    rng = np.random.default_rng(0)
    np.savez(tmp_path / "small.npz", dynamics_W1=rng.normal(size=(32, 6)), dynamics_b1=np.zeros(32),
             dynamics_W2=rng.normal(size=(4, 32)), dynamics_b2=np.zeros(4))
    with pytest.raises(ValueError, match="layers"):
        nn_io.load(tmp_path / "small.npz")
    np.savez(tmp_path / "other.npz", weights=np.zeros(3))
    with pytest.raises(ValueError, match="neither"):
        nn_io.load(tmp_path / "other.npz")
