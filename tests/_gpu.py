"""Device-memory plumbing for the GPU tests (torch tensors as CUDA buffers; the engine itself does not use torch)."""
import ctypes as C

import numpy as np


def torch():
    import torch as _t

    if not _t.cuda.is_available():
        raise RuntimeError("GPU tests need CUDA")
    return _t


def dev(a) -> "torch.Tensor":
    t = torch()
    return t.from_numpy(np.ascontiguousarray(a)).cuda()


def empty(n, dtype="float32"):
    t = torch()
    return t.empty(int(n), dtype=getattr(t, dtype), device="cuda")


def ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def stream() -> C.c_void_p:
    return C.c_void_p(torch().cuda.current_stream().cuda_stream or None)


def host(t) -> np.ndarray:
    torch().cuda.synchronize()
    return t.cpu().numpy()
