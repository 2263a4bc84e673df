"""The allocation-free update entry point (mppi_kernel_weighted_reduction_noalloc) against the allocating one.

It exists for callers that may not allocate GPU memory once running (frozen memory map in a real-time loop, memory
owned by another allocator, allocation banned after start-up); its scratch is a fixed array in the library's device
image.  The file sorts last so a stop-at-first-failure run has executed every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from mppi_generic_vendor_gb300 import _abi as A
from tests._gpu import dev, empty, host, ptr, stream

pytestmark = pytest.mark.gpu


def _case(K, T, Cd, seed):
    rng = np.random.default_rng(seed)
    w = np.exp(-rng.gamma(2.0, 3.0, K)).astype(np.float32)
    u = rng.normal(0.0, 1.0, K * T * Cd).astype(np.float32)
    norm = np.float32(w.astype(np.float64).sum())
    return w, u, np.array([0.0, norm], np.float32)


@pytest.mark.parametrize("K,T,Cd", [(2048, 100, 1), (5000, 64, 2), (3000, 50, 3), (1500, 40, 4),
                                    (65536, 256, 4)])
def test_noalloc_matches_allocating_entry_point_twice(K, T, Cd):
    """Both entry points run the same reduction kernel with the same 128-sample chunks, so the results are equal bit
    for bit; (65536, 256, 4) is the documented limit (512 chunks, 2 MiB of partial sums in the fixed array)."""
    w, u, bn = _case(K, T, Cd, K + T)
    wd, ud, bnd = dev(w), dev(u), dev(bn)
    ref = empty(T * Cd)
    A.call("mppi_kernel_weighted_reduction", ptr(wd), ptr(ud), ptr(ref), ptr(bnd), 0, T, K, Cd, stream())
    expect = host(ref)
    for _ in range(2):  # the scratch keeps the previous call's contents; the second call must not depend on them
        out = empty(T * Cd)
        A.call("mppi_kernel_weighted_reduction_noalloc", ptr(wd), ptr(ud), ptr(out), ptr(bnd), 0, T, K, Cd, stream())
        got = host(out)
        assert np.array_equal(got.view(np.uint32), expect.view(np.uint32))


def test_noalloc_rejects_sizes_beyond_its_scratch():
    w, u, bn = _case(256, 4, 1, 1)
    wd, ud, bnd, out = dev(w), dev(u), dev(bn), empty(4)
    st = A.lib().mppi_kernel_weighted_reduction_noalloc(ptr(wd), ptr(ud), ptr(out), ptr(bnd), 0, 4, 70000, 1,
                                                        stream())
    assert st == 1 and b"allocation-free limit" in A.lib().mppi_last_error_string()
    st = A.lib().mppi_kernel_weighted_reduction_noalloc(ptr(wd), ptr(ud), ptr(out), ptr(bnd), 0, 600, 256, 2,
                                                        stream())
    assert st == 1 and b"allocation-free limit" in A.lib().mppi_last_error_string()
