"""Fused elementwise chains with row outputs, against the builtins they fuse.

A `(map E1 E2 ...)` chain writes one value per row and expression, a
`(compress MASK E1 E2 ...)` chain the rows where MASK holds; both must give
exactly what the builtin statements give (the autofusion rewrite,
optimizer/autofusion.cc:770-935, does not change results).  Sizes cover the
empty input, one row (an inline result), a tail shorter than one round of
the kernel's unrolled rows, and tens of millions of rows; a division by zero
inside a chain is reported like the builtin's.
"""
import numpy as np
import pytest

from horsepower_gb300.abi import H_B, H_E, H_I, BuiltinError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import horsepower_gb300
    return horsepower_gb300.load()


def _np(L, z):
    return np.asarray(L.to_py(z))


@pytest.mark.parametrize("n", [0, 1, 7, 1_000_003, 15_000_000])
def test_map_filter_equals_statements(gpu, n):
    from horsepower_gb300 import plans as P
    rng = np.random.default_rng(61)
    date = rng.integers(8000, 10500, n).astype(np.int32)
    x = gpu.vec(date, H_I)
    lo, hi = 8766, 9131
    ch = P.Chain(gpu, f"(map (and (geq x0 {lo}:i32) (lt x0 {hi}:i32)))")
    fused = _np(gpu, ch.run([x]))
    d1 = gpu.call("pfnGeq", x, gpu.scalar(lo, H_I))
    d2 = gpu.call("pfnLt", x, gpu.scalar(hi, H_I))
    plain = _np(gpu, gpu.call("pfnAnd", d1, d2))
    assert fused.dtype == plain.dtype and fused.tobytes() == plain.tobytes()
    assert np.array_equal(fused, (date >= lo) & (date < hi))
    gpu.free_inputs()


@pytest.mark.parametrize("n", [1, 5, 2_000_001])
def test_map_several_outputs(gpu, n):
    from horsepower_gb300 import plans as P
    rng = np.random.default_rng(62)
    a = rng.standard_normal(n)
    b = rng.integers(-50, 50, n).astype(np.int32)
    xa, xb = gpu.vec(a, H_E), gpu.vec(b, H_I)
    ch = P.Chain(gpu, "(map (mul x0 x1) (plus x1 7:i32) (lt x0 0.25:f64))")
    z = [_np(gpu, v) for v in ch.run_many([xa, xb], 3)]
    want = [_np(gpu, gpu.call("pfnMul", xa, xb)), _np(gpu, gpu.call("pfnPlus", xb, gpu.scalar(7, H_I))),
            _np(gpu, gpu.call("pfnLt", xa, gpu.scalar(0.25, H_E)))]
    for g, w in zip(z, want):
        assert g.dtype == w.dtype and g.tobytes() == w.tobytes()
    gpu.free_inputs()


@pytest.mark.parametrize("n", [0, 3, 6_001_215])
def test_compress_chain_equals_statements(gpu, n):
    from horsepower_gb300 import plans as P
    rng = np.random.default_rng(63)
    qty = rng.integers(1, 51, n).astype(np.int32)
    price = rng.uniform(900, 105000, n)
    xq, xp = gpu.vec(qty, H_I), gpu.vec(price, H_E)
    ch = P.Chain(gpu, "(compress (lt x0 24:i32) x1 (mul x1 x0))")
    z = [_np(gpu, v) for v in ch.run_many([xq, xp], 2)]
    m = gpu.call("pfnLt", xq, gpu.scalar(24, H_I))
    want = [_np(gpu, gpu.call("pfnCompress", m, xp)),
            _np(gpu, gpu.call("pfnCompress", m, gpu.call("pfnMul", xp, xq)))]
    for g, w in zip(z, want):
        assert g.dtype == w.dtype and g.tobytes() == w.tobytes()
    gpu.free_inputs()


def test_map_division_by_zero_is_reported(gpu):
    from horsepower_gb300 import plans as P
    a = np.arange(1, 100_001, dtype=np.int32)
    b = np.ones(100_000, dtype=np.int32)
    b[77_777] = 0
    xa, xb = gpu.vec(a, H_I), gpu.vec(b, H_I)
    ch = P.Chain(gpu, "(map (div x0 x1))")
    with pytest.raises(BuiltinError) as chain_err:
        ch.run([xa, xb])
    with pytest.raises(BuiltinError) as plain_err:
        gpu.call("pfnDiv", xa, xb)
    assert chain_err.value.code == plain_err.value.code
    # the library stays usable
    ok = _np(gpu, ch.run([xa, gpu.vec(np.ones(100_000, dtype=np.int32), H_I)]))
    assert np.array_equal(ok, a)
    gpu.free_inputs()
