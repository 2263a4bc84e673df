"""The C-ABI library loads, exports every symbol include/mppi_gb.h declares, and rejects bad arguments on the host
before touching the GPU (the reference exits the process instead: gpu_err_chk.cuh:32-40, mppi_common.cu:1302-1313)."""
import ctypes as C
import re

import numpy as np
import pytest

from mppi_generic_vendor_gb300 import _abi as A


def declared_functions():
    text = A.HEADER_PATH.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mppi_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported_and_bound():
    lib = A.lib()
    names = declared_functions()
    assert len(names) > 30
    bound = {n for n, _, _ in A.SIGNATURES}
    for n in names:
        assert hasattr(lib, n), f"{n} declared in mppi_gb.h but not exported"
        assert n in bound, f"{n} has no ctypes signature"
    assert lib.mppi_abi_version() == 3


@pytest.mark.parametrize("model", [A.MODEL_CARTPOLE, A.MODEL_DOUBLE_INTEGRATOR, A.MODEL_BICYCLE_COSTMAP,
                                   A.MODEL_BICYCLE_SLIP, A.MODEL_BICYCLE_SLIP_MLP])
def test_param_block_sizes_match_header(model):
    d, c = C.c_size_t(), C.c_size_t()
    A.call("mppi_model_param_sizes", model, C.byref(d), C.byref(c))
    dt, ct = A.MODEL_PARAM_TYPES[model]
    assert d.value == C.sizeof(dt) and c.value == C.sizeof(ct)
    s, cd, o = C.c_int(), C.c_int(), C.c_int()
    A.call("mppi_model_dims", model, C.byref(s), C.byref(cd), C.byref(o))
    assert s.value in (4, 7) and cd.value in (1, 2) and o.value == s.value


def test_reference_defaults():
    sp = A.default_sampling_params()
    # GaussianParamsImpl defaults (gaussian.cuh:21-41); ColoredNoiseParamsImpl (colored_noise.cuh:44-50)
    assert list(sp.std_dev) == [1.0] * 4 and list(sp.control_cost_coeff) == [0.0] * 4
    assert sp.pure_noise_trajectories_percentage == np.float32(0.01) and sp.std_dev_decay == 1.0
    assert sp.offset_decay_rate == np.float32(0.97) and sp.fmin == 0.0
    cc = A.default_constraints()  # setDefaultControlRanges (dynamics.cu:19-26)
    assert cc.lower[0] == -np.finfo(np.float32).max and cc.upper[0] == np.finfo(np.float32).max
    cp = A.default_controller_params()  # ControllerParams (controller.cuh:46-68)
    assert cp.lambda_ == 1.0 and cp.alpha == 0.0 and cp.num_iters == 1


def test_defaults_without_the_library_equal_the_library_defaults():
    """The CPU baseline fills its parameter blocks without mapping libmppi_gb.so; the values must be the same."""
    for f in (A.default_controller_params, A.default_sampling_params, A.default_constraints):
        assert bytes(f(native=False)) == bytes(f()), f.__name__


def _create(model=A.MODEL_CARTPOLE, K=(64,), T=(16,), dyn_bytes=None, **over):
    cp = A.default_controller_params()
    sp = A.default_sampling_params()
    for k, v in over.items():
        setattr(cp if hasattr(cp, k) else sp, k, v)
    dt, ct = A.MODEL_PARAM_TYPES.get(model, A.MODEL_PARAM_TYPES[A.MODEL_CARTPOLE])
    n = len(K)
    dyn = (dt * n)()
    cost = (ct * n)()
    Ka = (C.c_int * n)(*K)
    Ta = (C.c_int * n)(*T)
    h = C.c_void_p()
    st = A.lib().mppi_create(model, n, Ka, Ta, C.byref(cp), C.byref(sp), None, C.cast(dyn, C.c_void_p),
                             dyn_bytes or C.sizeof(dt), C.cast(cost, C.c_void_p), C.sizeof(ct), None,
                             None, C.byref(h))
    return st, h


@pytest.mark.parametrize("kwargs", [dict(K=(0,)), dict(T=(0,)), dict(num_iters=0), dict(lambda_=0.0),
                                    dict(lambda_=-1.0), dict(dyn_bytes=3), dict(model=99),
                                    dict(pure_noise_trajectories_percentage=2.0), dict(kind=7)])
def test_create_rejects_bad_arguments_without_gpu(kwargs):
    st, h = _create(**kwargs)
    assert st == 1, A.STATUS_NAMES.get(st)
    assert not h.value
    assert A.lib().mppi_last_error_string()


def test_calls_on_null_handle_fail_cleanly():
    lib = A.lib()
    out = np.zeros(4, np.float32)
    assert lib.mppi_compute_control(None, out.ctypes.data_as(C.POINTER(C.c_float)), 1) == 1
    assert lib.mppi_get_control_seq(None, out.ctypes.data_as(C.POINTER(C.c_float))) == 1
    assert lib.mppi_destroy(None) == 0
    assert b"invalid handle" in lib.mppi_last_error_string()


def test_kernel_entries_reject_null_pointers_without_gpu():
    lib = A.lib()
    assert lib.mppi_kernel_weight_transform(None, None, 1.0, 16, 1, None) == 1
    assert lib.mppi_kernel_weighted_reduction(None, None, None, None, 0, 4, 4, 1, None) == 1
    assert lib.mppi_kernel_philox_normal(None, 4, 0, 0, None) == 1


def test_cpp_mirror_header_compiles():
    """include/mppi_gb.hpp (the C++ host mirror) compiles warning-free against include/mppi_gb.h (no GPU needed)."""
    import shutil
    import subprocess
    from pathlib import Path

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    root = Path(__file__).resolve().parents[1]
    subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                    str(root / "tests" / "cpp" / "cartpole_mirror.cpp"), "-I", str(root / "include")], check=True)


def _reference_top_scan(w, n):
    """controller.cu:126-181 restated: first n indices, then every later weight strictly above the list's current
    minimum (first minimum in list order) replaces it."""
    idx = list(range(n))

    def find_min():
        mi, mv = 0, w[idx[0]]
        for s in range(1, n):
            if w[idx[s]] < mv:
                mi, mv = s, w[idx[s]]
        return mi, mv

    mi, mv = find_min()
    for k in range(n, len(w)):
        if w[k] > mv:
            idx[mi] = k
            mi, mv = find_min()
    return idx


@pytest.mark.parametrize("K,n,ties", [(1, 1, False), (50, 5, False), (1000, 17, False), (300, 10, True),
                                      (64, 64, False)])
def test_select_top_samples_matches_reference_scan(K, n, ties):
    """mppi_select_top_samples (host only) picks the same indices, in the same slot order, as the reference's scan,
    and they are the n largest weights."""
    from mppi_generic_vendor_gb300 import select_top_samples

    rng = np.random.default_rng(K + n)
    w = rng.exponential(1.0, K).astype(np.float32)
    if ties:
        w = np.round(w * 4.0).astype(np.float32) / 4.0  # many equal weights
    got = select_top_samples(w, n)
    assert got.tolist() == _reference_top_scan(w.tolist(), n)
    assert np.array_equal(np.sort(w[got]), np.sort(w)[-n:])


def test_select_top_samples_rejects_bad_arguments():
    from mppi_generic_vendor_gb300 import select_top_samples

    with pytest.raises(A.MPPIError):
        select_top_samples(np.ones(4, np.float32), 5)
    with pytest.raises(A.MPPIError):
        select_top_samples(np.ones(4, np.float32), 0)


def test_fp8_quantisation_host_only():
    """mppi_mlp_quantize runs on the host: E4M3 weights with one power-of-two scale per layer (the smallest with
    max |W| / scale <= 448), so q * scale is exact in FP16 and FP32; BF16 keeps the weights and scale 1."""
    rng = np.random.default_rng(3)
    p = np.zeros(A.MLP_PARAMS, np.float32)
    p[:A.MLP_WEIGHTS] = rng.normal(0.0, 0.3, A.MLP_WEIGHTS).astype(np.float32)
    p[A.MLP_WEIGHTS + 9:A.MLP_WEIGHTS + 18] = 1.0  # input scales
    q = np.empty(A.MLP_PARAMS, np.float32)
    sc = np.empty(3, np.float32)
    fp = C.POINTER(C.c_float)
    A.call("mppi_mlp_quantize", p.ctypes.data_as(fp), 1, q.ctypes.data_as(fp), sc.ctypes.data_as(fp))
    for l, (lo, hi) in enumerate([(0, 576), (640, 4736), (4800, 5120)]):
        m, e = np.frexp(sc[l])
        assert m == 0.5
        assert np.abs(p[lo:hi]).max() / sc[l] <= 448.0 < 2.0 * np.abs(p[lo:hi]).max() / sc[l]
        w = q[lo:hi] * sc[l]
        assert np.array_equal(w.astype(np.float16).astype(np.float32), w)
        assert np.abs(w - p[lo:hi]).max() <= 2.0 ** -4 * np.abs(p[lo:hi]).max()
    A.call("mppi_mlp_quantize", p.ctypes.data_as(fp), 0, q.ctypes.data_as(fp), sc.ctypes.data_as(fp))
    assert np.array_equal(q, p) and np.array_equal(sc, np.ones(3, np.float32))
