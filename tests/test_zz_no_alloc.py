"""The allocation-free sum entry point agrees with pfnSum.

hgpuSumF64Static exists for callers that cannot allocate device memory where
they need a sum (inside a stream capture, under a fixed memory budget, or on
a path that cannot take an allocation's synchronisation); it keeps its tile
partials in a static device array.  The test calls it through the C ABI,
twice in a row on the same static array, and compares both results with the
arena-based pfnSum bit for bit (both sum the same fixed-point tiles).  This
file is collected last so a failure here never hides the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from horsepower_gb300.abi import H_E, V0

pytestmark = pytest.mark.gpu


def test_static_sum_matches_pfnsum_twice():
    import horsepower_gb300
    L = horsepower_gb300.load()
    fn = L.lib.hgpuSumF64Static
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    L.lib.hgpuStream.restype = C.c_void_p
    rng = np.random.default_rng(99)
    for n in (20_000_003, 4096 * 5 + 17):
        x = rng.uniform(0, 1e5, n)
        expect = L.to_py(L.call("pfnSum", L.vec(x, H_E)))[0]
        dx, dout = V0(), V0()  # the test allocates the input and the output; the entry point does not
        assert L.lib.hgpuToDevice(C.byref(dx), C.byref(L.vec(x, H_E))) == 0
        assert L.lib.hgpuToDevice(C.byref(dout), C.byref(L.vec(np.full(2, -1.0), H_E))) == 0
        assert L.lib.hgpuSync() == 0
        for _ in range(2):
            rc = fn(dx.g, n, dout.g, L.lib.hgpuStream())
            assert rc == 0, L.lib.hgpuLastError()
            assert L.lib.hgpuSync() == 0
            got = L.to_py(dout)[0]
            assert got == expect, (got, expect)  # the same fixed-point tiles as pfnSum: the same bits
        L.free_inputs()


def test_static_sum_rejects_oversize():
    import horsepower_gb300
    L = horsepower_gb300.load()
    fn = L.lib.hgpuSumF64Static
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    rc = fn(None, 65536 * 4096 + 1, None, None)
    assert rc == 5  # E_LENGTH, before touching any memory
    assert b"outside" in L.lib.hgpuLastError()
