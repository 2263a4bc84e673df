"""mppi_ddp_feedback_gains (the handle-free DDP feedback solver) for the tests, and the feedback control in the
engine's FP32 order."""
import ctypes as C

import numpy as np

from mppi_generic_vendor_gb300 import _abi as A


def _fp(a):
    return np.ascontiguousarray(a, dtype=np.float32).ctypes.data_as(C.POINTER(C.c_float))


def engine_gains(model, dyn, x0, xt, un, dt, Q=None, Qf=None, R=None, iterations=1, lo=None, hi=None):
    """mppi_ddp_feedback_gains as (H, C, S) arrays; the weights go in column-major like the reference's Eigen."""
    H, S = xt.shape
    Cd = un.shape[1]
    lo = np.full(Cd, -1e30, np.float32) if lo is None else np.asarray(lo, np.float32)
    hi = np.full(Cd, 1e30, np.float32) if hi is None else np.asarray(hi, np.float32)
    keep = [np.ascontiguousarray(np.asarray(m, np.float32).T) if m is not None else None for m in (Q, Qf, R)]
    out = np.zeros(H * Cd * S, np.float32)
    args = [np.ascontiguousarray(a, np.float32) for a in (x0, xt, un, lo, hi)]
    st = A.lib().mppi_ddp_feedback_gains(model, C.cast(C.pointer(dyn), C.c_void_p), C.sizeof(dyn), H, dt,
                                         _fp(args[0]), _fp(args[1]), _fp(args[2]),
                                         *[None if m is None else _fp(m) for m in keep], int(iterations),
                                         _fp(args[3]), _fp(args[4]), out.ctypes.data_as(C.POINTER(C.c_float)))
    return st, out.reshape(H, S, Cd).transpose(0, 2, 1)


def feedback_control(K, x, goal):
    """K (C, S) applied to x - goal in FP32, each control's products added in state order (DDPFeedback::k_)."""
    out = np.zeros(K.shape[0], np.float32)
    for r in range(K.shape[0]):
        acc = np.float32(0.0)
        for c in range(K.shape[1]):
            acc = np.float32(acc + np.float32(np.float32(K[r, c]) * np.float32(np.float32(x[c]) - np.float32(goal[c]))))
        out[r] = acc
    return out
