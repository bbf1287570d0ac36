"""The allocation-free sum entry point agrees with pfnSum and allocates nothing.

hgpuSumF64Static exists for callers that cannot allocate device memory where
they need a sum: an engine held to a device-memory budget it reserved up
front, or a latency path that cannot take the synchronisation an allocation
may cause.  It keeps its tile partials in a static device array.  The test
calls it through the C ABI, twice in a row on the same static array, and
compares both results with the arena-based pfnSum bit for bit (both sum the
same fixed-point tiles).  Across each call the device's free memory (as
cudaMemGetInfo reports it) and the output arena's offset stay the same.  The
sizes cover the empty vector (a memset of the result), one tile written
straight into the result, two tiles, three reduction levels and the largest
accepted n.  This file is collected last so a failure here never hides the
other tests.
"""
import ctypes as C

import numpy as np
import pytest

from horsepower_gb300.abi import H_E, V0

pytestmark = pytest.mark.gpu

MAX_ROWS = 65536 * 4096


def _bind(L):
    fn = L.lib.hgpuSumF64Static
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    L.lib.hgpuStream.restype = C.c_void_p
    L.lib.getHeapOffset.restype = C.c_longlong
    return fn


def _free_bytes():
    rt = C.CDLL("libcudart.so.13")  # the runtime libhgpu already loaded: same context
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("n", [0, 1, 4096, 4097, 4096 * 5 + 17, 20_000_003, MAX_ROWS])
def test_static_sum_matches_pfnsum_twice(n):
    import horsepower_gb300
    L = horsepower_gb300.load()
    fn = _bind(L)
    rng = np.random.default_rng(99 + n % 1000)
    x = rng.uniform(0, 1e5, n) if n < MAX_ROWS else np.full(n, 0.1) + np.arange(n) % 7
    expect = L.to_py(L.call("pfnSum", L.vec(x, H_E)))[0]
    dx, dout = V0(), V0()  # the test allocates the input and the output; the entry point does not
    assert L.lib.hgpuToDevice(C.byref(dx), C.byref(L.vec(x if n else np.zeros(2), H_E))) == 0
    assert L.lib.hgpuToDevice(C.byref(dout), C.byref(L.vec(np.full(2, -1.0), H_E))) == 0
    assert L.lib.hgpuSync() == 0
    assert fn(dx.g, min(n, 4096), dout.g, L.lib.hgpuStream()) == 0  # first call on the device: address look-up
    assert L.lib.hgpuSync() == 0
    for _ in range(2):
        heap0, free0 = L.lib.getHeapOffset(), _free_bytes()
        rc = fn(dx.g, n, dout.g, L.lib.hgpuStream())
        assert rc == 0, L.lib.hgpuLastError()
        assert L.lib.hgpuSync() == 0
        assert L.lib.getHeapOffset() == heap0, "the call moved the output arena"
        assert _free_bytes() == free0, "device memory was allocated during the call"
        got = L.to_py(dout)[0]
        assert got == expect, (got, expect)  # the same fixed-point tiles as pfnSum: the same bits
    L.free_inputs()


def test_static_sum_rejects_oversize():
    import horsepower_gb300
    L = horsepower_gb300.load()
    fn = _bind(L)
    rc = fn(None, MAX_ROWS + 1, None, None)
    assert rc == 5  # E_LENGTH, before touching any memory
    assert b"outside" in L.lib.hgpuLastError()
    assert fn(None, -1, None, None) == 5
