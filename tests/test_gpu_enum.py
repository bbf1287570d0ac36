"""Enum / foreign-key path on the GPU: pfnEnum, pfnValues, pfnKeys, pfnFetch
(h_primitive.cc:191-225, 2198-2222) at the sizes of a foreign key into a
15M-row key column, against the oracle port and through size-independent
properties: gathering the key column through the enum's index gives the
foreign-key column back, and a foreign key with no key is E_ENUM_INDEX.
"""
import ctypes as C
import os

import numpy as np
import pytest

from horsepower_gb300.abi import Builtins, H_B, H_D, H_I, H_L, H_Y
from horsepower_gb300 import batch as B

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
E_ENUM_INDEX, E_NOT_IMPL = 10, 99


@pytest.fixture(scope="module")
def libs():
    import subprocess
    import horsepower_gb300
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return horsepower_gb300.load(), Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")


def enum_outputs(L, x, y, pmask):
    e = L.call("pfnEnum", x, y)
    assert e.typ == H_Y and e.len == y.len
    idx = L.call("pfnValues", e)
    return e, [L.to_py(idx), L.to_py(L.call("pfnFetch", e)), L.to_py(L.call("pfnKeys", e)),
               L.to_py(L.call("pfnIndex", pmask, idx))]


@pytest.mark.parametrize("kind", ["permutation_i32", "sorted_sparse_i64", "dup_keys_i64"])
def test_enum_matches_oracle(libs, kind):
    rng = np.random.default_rng(5)
    nk, nf = 2_000_000, 6_000_000
    if kind == "permutation_i32":
        pk, typ = rng.permutation(nk).astype(np.int32), H_I
    elif kind == "sorted_sparse_i64":
        pk, typ = (np.arange(nk, dtype=np.int64) * 4 + 1), H_L
    else:  # repeated keys: the first occurrence wins (hash path)
        pk, typ = rng.integers(0, nk // 3, nk).astype(np.int64), H_L
    fk = pk[rng.integers(0, nk, nf)]
    pm = rng.random(nk) < 0.4
    outs = []
    for L in libs:
        x, y, m = L.vec(pk, typ), L.vec(fk, typ), L.vec(pm, H_B)
        outs.append(enum_outputs(L, x, y, m)[1])
    for a, b in zip(*outs):
        assert a.dtype == b.dtype and np.array_equal(a, b)
    idx = outs[0][0]
    assert np.array_equal(pk[idx], fk)
    if kind != "dup_keys_i64":
        assert np.array_equal(outs[0][3], pm[idx])


def test_enum_full_size_round_trip(libs):
    """A 60M-row foreign key into a 15M-row permuted key column, device resident."""
    gpu = libs[0]
    rng = np.random.default_rng(6)
    nk, nf = 15_000_000, 60_000_000
    pk = rng.permutation(nk).astype(np.int32)
    fk = pk[rng.integers(0, nk, nf)]
    x, y = B.to_device(gpu, pk, H_I), B.to_device(gpu, fk, H_I)
    e = gpu.call("pfnEnum", x, y)
    idx = gpu.to_py(gpu.call("pfnValues", e))
    assert idx.dtype == np.int64 and np.array_equal(pk[idx], fk)
    # the gather through the enum (no bounds check needed) equals the foreign keys
    back = gpu.to_py(gpu.call("pfnIndex", x, gpu.call("pfnValues", e)))
    assert np.array_equal(back, fk)
    # one foreign key without a key, first or last row: E_ENUM_INDEX
    for pos in (0, nf - 1):
        bad = fk.copy()
        bad[pos] = nk + 7
        assert gpu.rc("pfnEnum", x, B.to_device(gpu, bad, H_I)) == E_ENUM_INDEX
    gpu.free_inputs()


def test_enum_sorted_full_size(libs):
    """Sorted sparse 64-bit keys (the layout of an order key): binary search path."""
    gpu = libs[0]
    rng = np.random.default_rng(7)
    nk, nf = 15_000_000, 60_000_000
    pk = np.arange(nk, dtype=np.int64) * 4 + 1
    pos = rng.integers(0, nk, nf)
    x, y = B.to_device(gpu, pk, H_L), B.to_device(gpu, pk[pos], H_L)
    e = gpu.call("pfnEnum", x, y)
    assert np.array_equal(gpu.to_py(gpu.call("pfnValues", e)), pos)
    gpu.free_inputs()


def test_enum_edges(libs):
    for L in libs:
        x = L.vec(np.array([5, 9, 2], np.int32), H_I)
        one = L.call("pfnEnum", x, L.vec(np.array([9], np.int32), H_I))
        assert one.len == 1 and L.to_py(L.call("pfnValues", one)).tolist() == [1]
        empty = L.call("pfnEnum", x, L.vec(np.zeros(0, np.int32), H_I))
        assert empty.len == 0 and L.to_py(L.call("pfnValues", empty)).size == 0
        assert L.call("pfnLen", one).i64 == 1
        # @compress of an enum stops the reference process (TODO at h_primitive.cc:1492): an error here
        assert L.rc("pfnCompress", L.vec(np.array([True]), H_B), one) == E_NOT_IMPL
        assert L.rc("pfnFetch", x) == 1 and L.rc("pfnValues", x) == 1
        # dates hash as 32-bit integers; a date foreign key into a date key column
        d = L.vec(np.array([9000, 9003, 9001], np.int32), H_D)
        ed = L.call("pfnEnum", d, L.vec(np.array([9001, 9000, 9001], np.int32), H_D))
        assert L.to_py(L.call("pfnValues", ed)).tolist() == [2, 0, 2]
        assert L.rc("pfnEnum", d, L.vec(np.array([9002], np.int32), H_D)) == E_ENUM_INDEX
        L.free_inputs()


def test_enum_host_residency(libs):
    gpu = libs[0]
    rng = np.random.default_rng(8)
    pk = rng.permutation(50_000).astype(np.int64)
    fk = pk[rng.integers(0, 50_000, 200_000)]
    gpu.lib.hgpuSetResidency(1)
    try:
        x, y = gpu.vec(pk, H_L), gpu.vec(fk, H_L)
        e = gpu.call("pfnEnum", x, y)
        assert not gpu.lib.hgpuIsDevice(C.byref(e))
        idx = gpu.call("pfnValues", e)
        # the index is host memory the caller can read directly
        raw = np.frombuffer((C.c_char * (8 * idx.len)).from_address(idx.g), np.int64)
        assert np.array_equal(pk[raw], fk)
    finally:
        gpu.lib.hgpuSetResidency(0)
        gpu.free_inputs()


@pytest.mark.parametrize("dist", ["uniform_wide", "clustered", "dense_tail", "dense_negative"])
def test_index_of_strictly_increasing_matches_oracle(libs, dist):
    """Sorted unique keys take the rank table (range under 8 per key) or the
    bucket-table search on the GPU; the oracle restates the reference's
    recursive binary search."""
    rng = np.random.default_rng(9)
    n = 3_000_000
    if dist == "dense_negative":  # rank table
        x = np.unique(rng.integers(-5 * n, 2 * n, n))
    elif dist == "uniform_wide":
        x = np.unique(rng.integers(-2 ** 62, 2 ** 62, n))
    elif dist == "clustered":  # most keys in a few narrow clusters, huge empty gaps
        x = np.unique(np.concatenate([rng.integers(c, c + 4 * n, n // 4) for c in (-2 ** 60, 0, 2 ** 40, 2 ** 61)]))
    else:  # dense run then a few far keys: most buckets empty
        x = np.concatenate([np.arange(n, dtype=np.int64), [2 ** 50, 2 ** 55, 2 ** 62]])
    x = x.astype(np.int64)
    y = np.concatenate([x[rng.integers(0, x.size, 4_000_000)], rng.integers(-2 ** 63, 2 ** 63 - 1, 1_000_000),
                        x[:3] - 1, x[-3:] + 1]).astype(np.int64)
    rng.shuffle(y)
    outs = [L.to_py(L.call("pfnIndexOf", L.vec(x, H_L), L.vec(y, H_L))) for L in libs]
    assert np.array_equal(outs[0], outs[1])
    hit = outs[0] < x.size
    assert np.array_equal(x[outs[0][hit]], y[hit])
    for L in libs:
        L.free_inputs()


def test_index_of_ordered_reads_probes_at_key_width(libs):
    """An ordered key column is searched with y read at x's width
    (h_system.cc:735-742): i64 or f64 probes under i32 keys are read as 32-bit
    words; probes narrower than the keys are an error (the reference reads past
    their end)."""
    rng = np.random.default_rng(10)
    x32 = np.unique(rng.integers(0, 1 << 20, 5000)).astype(np.int32)
    y64 = rng.integers(0, 1 << 20, 3000).astype(np.int64)
    yf = rng.standard_normal(300)
    for ytyp, yv in ((H_L, y64), (6, yf)):
        outs = [L.to_py(L.call("pfnIndexOf", L.vec(x32, H_I), L.vec(yv, ytyp))) for L in libs]
        assert np.array_equal(outs[0], outs[1])
    x64 = np.arange(0, 4000, 2, dtype=np.int64)
    for L in libs:
        assert L.rc("pfnIndexOf", L.vec(x64, H_L), L.vec(y64.astype(np.int32), H_I)) == 6
        assert L.rc("pfnIndexOf", L.vec(x32, H_I), L.vec(y64.astype(np.int16), 2)) == 6
        # unordered keys hash with promotion: narrower probes are fine
        assert L.rc("pfnIndexOf", L.vec(rng.permutation(x64), H_L), L.vec(y64.astype(np.int32), H_I)) == 0
        L.free_inputs()
