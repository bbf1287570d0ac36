"""GPU parity against the oracle port on seeded inputs larger than the golden
fixtures, plus determinism and size-independent properties.

Bar: bit-exact for integer, index, boolean and permutation outputs; f64 sums
within a relative tolerance of 1e-12 of the oracle (whose OpenMP order, like
the reference's, depends on the thread count) and bit-exact against the
oracle's restatement of the library's fixed summation order.
"""
import ctypes as C
import os

import numpy as np
import pytest

from horsepower_gb300.abi import Builtins, H_B, H_C, H_E, H_I, H_L

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RTOL = 1e-12


@pytest.fixture(scope="module")
def libs():
    import subprocess
    import horsepower_gb300
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    ora = Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")
    for fn in (ora.lib.hgoTreeSumF64, ora.lib.hgoFixedSumF64):
        fn.restype = C.c_double
        fn.argtypes = [C.c_void_p, C.c_longlong]
    return horsepower_gb300.load(), ora


def both(libs, fn, mk):
    out = []
    for L in libs:
        z = L.call(fn, *mk(L))
        out.append(L.to_py(z))
        L.free_inputs()
    return out


def same(a, b):
    if isinstance(a, np.ndarray):
        return a.dtype == b.dtype and np.array_equal(a, b, equal_nan=a.dtype.kind == "f")
    if isinstance(a, tuple):
        return all(same(p, q) for p, q in zip(a[1:], b[1:]))
    return len(a) == len(b) and all(same(p, q) for p, q in zip(a, b))


@pytest.mark.parametrize("dens", [0.0, 0.018, 0.5, 1.0])
@pytest.mark.parametrize("typ,dt", [(H_E, np.float64), (H_I, np.int32), (H_B, np.bool_), (H_C, np.int8)])
def test_compress_large(libs, dens, typ, dt):
    rng = np.random.default_rng(11)
    n = 6_001_215
    m = rng.random(n) < dens
    v = rng.integers(-100, 100, n).astype(dt) if typ != H_E else rng.standard_normal(n)
    a, b = both(libs, "pfnCompress", lambda L: (L.vec(m, H_B), L.vec(v, typ)))
    assert same(a, b)


def test_where_large(libs):
    rng = np.random.default_rng(12)
    m = rng.random(10_000_001) < 0.3
    a, b = both(libs, "pfnWhere", lambda L: (L.vec(m, H_B),))
    assert same(a, b)


@pytest.mark.parametrize("fn", ["pfnLt", "pfnGeq", "pfnEq", "pfnMul", "pfnMinus", "pfnDiv", "pfnAnd"])
def test_elementwise_large(libs, fn):
    rng = np.random.default_rng(13)
    n = 5_000_003
    if fn == "pfnAnd":
        x, y, tx, ty = rng.random(n) < 0.5, rng.random(n) < 0.5, H_B, H_B
    else:
        x, y, tx, ty = np.round(rng.standard_normal(n), 3), rng.integers(1, 9, n).astype(np.int32), H_E, H_I
    a, b = both(libs, fn, lambda L: (L.vec(x, tx), L.vec(y, ty)))
    assert same(a, b)


def test_sum_deterministic_and_within_tolerance(libs):
    gpu, ora = libs
    rng = np.random.default_rng(14)
    x = rng.uniform(0, 1e5, 20_000_000)
    r1 = gpu.to_py(gpu.call("pfnSum", gpu.vec(x, H_E)))[0]
    r2 = gpu.to_py(gpu.call("pfnSum", gpu.vec(x, H_E)))[0]
    assert r1 == r2, "fixed-point tile sum is not reproducible"
    fixed = ora.lib.hgoFixedSumF64(x.ctypes.data, x.size)
    assert r1 == fixed, f"GPU sum {r1!r} != oracle restatement of the fixed-point tiles {fixed!r}"
    ref = ora.to_py(ora.call("pfnSum", ora.vec(x, H_E)))[0]
    assert abs(r1 - ref) <= RTOL * abs(ref)
    gpu.free_inputs()
    ora.free_inputs()


@pytest.mark.parametrize("kind", ["wide", "cancel", "subnormal", "huge", "tiny_tail", "specials"])
def test_sum_fixed_point_bit_exact(libs, kind):
    """f64 @sum/@avg: 128-bit fixed-point tiles, bit-exact against the oracle's
    restatement over 1 to 3 levels of tiles, and within 1e-12 of the reference
    order where the exact sum is not cancelled away."""
    gpu, ora = libs
    rng = np.random.default_rng(16)
    n = 17_000_001
    if kind == "wide":
        x = rng.standard_normal(n) * np.ldexp(1.0, rng.integers(-200, 200, n))
    elif kind == "cancel":
        x = rng.standard_normal(n)
        x = np.concatenate([x, -x[::-1]])
    elif kind == "subnormal":
        x = rng.standard_normal(n) * 1e-310
    elif kind == "huge":  # partial sums past DBL_MAX: the exact tiles overflow only at the end
        x = np.full(n, 1.7976931348623157e308 / 3)
    elif kind == "tiny_tail":  # elements 2^100 below the largest binade of their tile
        x = np.where(rng.random(n) < 0.001, 1e30, rng.standard_normal(n))
    else:
        x = rng.standard_normal(n)
        x[[5, 9_000_000]] = [np.inf, np.inf]
    for fn in ("pfnSum", "pfnAvg"):
        got = gpu.to_py(gpu.call(fn, gpu.vec(x, H_E)))[0]
        want = ora.lib.hgoFixedSumF64(x.ctypes.data, x.size)
        if fn == "pfnAvg":
            want = want / x.size
        assert np.float64(got).tobytes() == np.float64(want).tobytes(), (fn, got, want)
        if kind in ("wide", "subnormal", "tiny_tail"):
            ref = ora.to_py(ora.call(fn, ora.vec(x, H_E)))[0]
            assert abs(got - ref) <= RTOL * abs(ref), (fn, got, ref)
    gpu.free_inputs()
    ora.free_inputs()


@pytest.mark.parametrize("typ", [H_E, 5])
def test_minmax_float_serial_fold_bits(libs, typ):
    """f64/f32 @min/@max follow the reference's serial fold bit for bit: the
    fold restarts after the last NaN, ends on a trailing NaN, and of equal
    values (-0.0 and +0.0) keeps the later one; sizes span several tile
    levels."""
    gpu, ora = libs
    rng = np.random.default_rng(17)
    dt = np.float64 if typ == H_E else np.float32
    n = 20_000_003
    pool = np.array([0.0, -0.0, 1.0, -1.0, 2.5, -2.5, np.inf, -np.inf], dt)
    base = pool[rng.integers(0, pool.size, n)]
    normal = rng.standard_normal(n).astype(dt)
    cases = [base, normal]
    for arr in (base, normal):
        for pos in ([17], [n // 2, n - 5000], [n - 1], [0, 4096 * 4096 + 3]):
            a = arr.copy()
            a[pos] = np.nan
            cases.append(a)
    cases.append(np.where(rng.random(n) < 0.5, dt(0.0), dt(-0.0)).astype(dt))
    for a in cases:
        for fn in ("pfnMin", "pfnMax"):
            g, o = both(libs, fn, lambda L: (L.vec(a, typ),))
            assert g.tobytes() == o.tobytes(), (fn, g, o)


@pytest.mark.parametrize("fn", ["pfnMin", "pfnMax", "pfnSum", "pfnAvg"])
def test_int_reductions_large(libs, fn):
    rng = np.random.default_rng(15)
    x = rng.integers(-2 ** 31, 2 ** 31 - 1, 9_000_001, dtype=np.int64).astype(np.int32)
    a, b = both(libs, fn, lambda L: (L.vec(x, H_I),))
    assert same(a, b) if fn != "pfnAvg" else abs(a[0] - b[0]) <= 1e-15 * abs(b[0])


def test_gather_large(libs):
    rng = np.random.default_rng(16)
    x = rng.standard_normal(3_000_000)
    idx = rng.integers(0, x.size, 8_000_000).astype(np.int64)
    a, b = both(libs, "pfnIndex", lambda L: (L.vec(x, H_E), L.vec(idx, H_L)))
    assert same(a, b)


def test_join_pk_fk(libs):
    rng = np.random.default_rng(17)
    D = 3_000_000
    pk = rng.permutation(D).astype(np.int32)
    keep = rng.random(D) < 0.15
    fk = rng.integers(0, D, 12_000_000).astype(np.int32)
    a, b = both(libs, "pfnJoinIndex", lambda L: (L.vec(pk[keep], H_I), L.vec(fk, H_I), L.sym("eq")))
    assert same(a, b)


def test_join_duplicates(libs):
    rng = np.random.default_rng(18)
    x = rng.integers(0, 20000, 200_000).astype(np.int32)
    y = rng.integers(0, 30000, 400_000).astype(np.int32)
    a, b = both(libs, "pfnJoinIndex", lambda L: (L.vec(x, H_I), L.vec(y, H_I), L.sym("eq")))
    assert same(a, b)


def test_index_of_and_member(libs):
    rng = np.random.default_rng(19)
    x = rng.permutation(4_000_000).astype(np.int64)[:1_000_000]
    y = rng.integers(0, 4_000_000, 5_000_000).astype(np.int64)
    a, b = both(libs, "pfnIndexOf", lambda L: (L.vec(x, H_L), L.vec(y, H_L)))
    assert same(a, b)
    a, b = both(libs, "pfnMember", lambda L: (L.vec(y, H_L), L.vec(x, H_L)))
    assert same(a, b)


@pytest.mark.parametrize("kind", ["i32", "i64_zipf", "trie", "list_li"])
def test_group_large(libs, kind):
    rng = np.random.default_rng(20)
    n = 3_000_000
    if kind == "i32":
        mk = lambda L: (L.vec(rng_a, H_I),)  # noqa: E731
        rng_a = rng.integers(-1000, 100000, n).astype(np.int32)
    elif kind == "i64_zipf":
        rng_a = np.minimum(rng.zipf(1.1, n), 1_000_000).astype(np.int64)
        mk = lambda L: (L.vec(rng_a, H_L),)  # noqa: E731
    elif kind == "trie":
        f, s = rng.integers(0, 3, n).astype(np.int8), rng.integers(0, 2, n).astype(np.int8)
        mk = lambda L: (L.list([L.vec(f, H_C), L.vec(s, H_C)]),)  # noqa: E731
    else:
        k, s = rng.integers(0, 5000, n).astype(np.int64), rng.integers(-3, 3, n).astype(np.int32)
        mk = lambda L: (L.list([L.vec(k, H_L), L.vec(s, H_I)]),)  # noqa: E731
    a, b = both(libs, "pfnGroup", mk)
    assert np.array_equal(a[1], b[1])
    assert len(a[2]) == len(b[2]) and all(np.array_equal(p, q) for p, q in zip(a[2], b[2]))


def test_order_key_sec(libs):
    rng = np.random.default_rng(21)
    n = 2_000_000
    key = np.minimum(rng.zipf(1.1, n), 10_000_000).astype(np.int64)
    sec = rng.integers(0, 2 ** 20 + 1, n).astype(np.int32)
    a, b = both(libs, "pfnOrderBy", lambda L: (L.list([L.vec(key, H_L), L.vec(sec, H_I)]), L.vec(np.array([1, 1], bool), H_B)))
    assert same(a, b)


@pytest.mark.parametrize("agg", ["hgpuGroupSum", "hgpuGroupAvg", "hgpuGroupMin", "hgpuGroupMax", "hgpuGroupLen"])
def test_group_aggregates_large(libs, agg):
    gpu, ora = libs
    rng = np.random.default_rng(22)
    n = 2_000_000
    key = np.minimum(rng.zipf(1.1, n), 200_000).astype(np.int64)
    pay = rng.uniform(0, 1e5, n)
    outs = []
    for L in libs:
        g = L.call("pfnGroup", L.vec(key, H_L))
        vals = L.call("pfnValues", g)
        outs.append(L.to_py(L.call(agg, L.vec(pay, H_E), vals)))
    a, b = outs
    assert a.dtype == b.dtype and a.shape == b.shape
    if agg in ("hgpuGroupSum", "hgpuGroupAvg"):
        assert np.allclose(a, b, rtol=RTOL, atol=0)
    else:
        assert np.array_equal(a, b)
    for L in libs:
        L.free_inputs()


def test_chain_equals_fused(libs):
    gpu, _ = libs
    rng = np.random.default_rng(23)
    key = rng.integers(0, 50_000, 1_000_000).astype(np.int32)
    pay = rng.uniform(0, 1e5, 1_000_000)
    g = gpu.call("pfnGroup", gpu.vec(key, H_I))
    vals = gpu.call("pfnValues", g)
    x = gpu.vec(pay, H_E)
    fused = gpu.to_py(gpu.call("hgpuGroupSum", x, vals))
    t = gpu.call("pfnEachRight", x, vals, gpu.fn_ptr("pfnIndex"))
    e = gpu.call("pfnEach", t, gpu.fn_ptr("pfnSum"))
    chain = gpu.to_py(gpu.call("pfnRaze", e))
    assert np.array_equal(fused, chain), "fused and chained group sums differ"
    gpu.free_inputs()


def test_fused_q6_chain(libs):
    """The q6 chain fused into one kernel equals the interpreter's plain
    builtin sequence (oracle) within 1e-12, and is reproducible."""
    from horsepower_gb300 import data as D, plans as P
    gpu, ora = libs
    t = D.filter_table()
    plain = ora.to_py(P.filter_aggregate(ora, P.host_nodes(ora, t, P.FILTER_TYPES)))[0]
    nodes = P.host_nodes(gpu, t, P.FILTER_TYPES)
    ch = P.Chain(gpu, P.Q6_CHAIN.format(lo=D.WIN_LO, hi=D.WIN_HI))
    f1 = gpu.to_py(ch.run([nodes["shipdate"], nodes["qty"], nodes["disc"], nodes["price"]]))[0]
    f2 = gpu.to_py(ch.run([nodes["shipdate"], nodes["qty"], nodes["disc"], nodes["price"]]))[0]
    assert f1 == f2
    assert abs(f1 - plain) <= RTOL * abs(plain), (f1, plain)
    gplain = gpu.to_py(P.filter_aggregate(gpu, nodes))[0]
    assert abs(gplain - plain) <= RTOL * abs(plain)
    gpu.free_inputs()
    ora.free_inputs()


def test_join_group_pipeline(libs):
    """The join + group-by query at 1/10 scale: GPU vs oracle."""
    from horsepower_gb300 import data as D, plans as P
    gpu, ora = libs
    dim, fact = D.join_tables(6_000_000, 1_500_000, seed=5)
    outs = []
    for L in libs:
        r = P.join_group(L, P.host_nodes(L, dim, P.DIM_TYPES), P.host_nodes(L, fact, P.FACT_TYPES))
        outs.append([L.to_py(v) for v in r])
        L.free_inputs()
    a, b = outs
    for k in (0, 1, 5):
        assert np.array_equal(a[k], b[k])
    for k in (2, 3, 4):
        assert np.allclose(a[k], b[k], rtol=RTOL, atol=0)


def test_join_group_async_uploads(libs):
    """The same query on columns uploaded with hgpuToDeviceAsync (copies on a
    second stream, builtins waiting per column) equals the synchronous
    upload, bit for bit, across heap rewinds that release the uploads."""
    import ctypes as C
    from horsepower_gb300 import data as D, plans as P
    from horsepower_gb300.abi import V0
    gpu, _ = libs
    dim, fact = D.join_tables(6_000_000, 1_500_000, seed=6)
    hd, hf = P.host_nodes(gpu, dim, P.DIM_TYPES), P.host_nodes(gpu, fact, P.FACT_TYPES)
    Lb = gpu.lib
    Lb.getHeapOffset.restype = C.c_longlong
    results = []
    for fn in (Lb.hgpuToDevice, Lb.hgpuToDeviceAsync, Lb.hgpuToDeviceAsync):
        mark = Lb.getHeapOffset()
        up = {}
        for part, nodes in (("dim", hd), ("fact", hf)):
            for k, v in nodes.items():
                z = V0()
                assert fn(C.byref(z), C.byref(v)) == 0
                up[(part, k)] = z
        r = P.join_group(gpu, {k: up[("dim", k)] for k in hd}, {k: up[("fact", k)] for k in hf})
        results.append([gpu.to_py(v) for v in r])
        Lb.setHeapOffset(C.c_longlong(mark))
    for other in results[1:]:
        for a, b in zip(results[0], other):
            assert a.dtype == b.dtype and np.array_equal(a, b)
    gpu.free_inputs()


@pytest.mark.parametrize("s", [0.05, 0.07, 0.0, -0.0, 1e-13, -1e-13, 5e-14, 24.0, 1e300, -1e300, 5e-324,
                               float("inf"), float("-inf"), float("nan"), 123456.789])
def test_compare_f64_scalar_edges(libs, s):
    """f64 compares against a scalar (either side) at compareFloat's 1e-13
    boundaries, signed zeros, infinities, NaN and denormals: bit-exact."""
    rng = np.random.default_rng(int(abs(s) * 1000) % 9973 if np.isfinite(s) else 7)
    base = 0.0 if not np.isfinite(s) else s
    v = [0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, s, np.nextafter(s, np.inf), np.nextafter(s, -np.inf)]
    v += [base + k * 2.5e-15 for k in range(-60, 61)] + [base + k * 1e-14 for k in range(-30, 31)]
    v += list(rng.standard_normal(2000) * 10.0 ** rng.integers(-20, 20, 2000))
    v = np.array(v * 3, dtype=np.float64)
    for fn in ("pfnLt", "pfnLeq", "pfnGt", "pfnGeq", "pfnEq", "pfnNeq"):
        a, b = both(libs, fn, lambda L: (L.vec(v, H_E), L.scalar(s, H_E)))
        assert same(a, b), (fn, "vs")
        a, b = both(libs, fn, lambda L: (L.scalar(s, H_E), L.vec(v, H_E)))
        assert same(a, b), (fn, "sv")


def test_unaligned_device_views(libs):
    """Device vectors that start at an odd element offset (views into another
    vector) take the unvectorised paths and give the same results."""
    from horsepower_gb300.abi import V0
    gpu, ora = libs
    rng = np.random.default_rng(44)
    n = 1_000_003
    m = rng.random(n + 1) < 0.3
    v = rng.standard_normal(n + 1)
    idx = np.sort(rng.integers(0, n, n // 3 + 1)).astype(np.int64)

    def dev_view(L, arr, typ, skip):
        h = L.vec(arr, typ)
        d = V0()
        assert L.lib.hgpuToDevice(C.byref(d), C.byref(h)) == 0
        L._keep.append(d)
        w = V0()
        w.typ, w.len, w.g = typ, arr.size - skip, d.g + skip * arr.itemsize
        L._keep.append(w)
        return w

    got = gpu.to_py(gpu.call("pfnCompress", dev_view(gpu, m, H_B, 1), dev_view(gpu, v, H_E, 1)))
    assert np.array_equal(got, v[1:][m[1:]])
    got = gpu.to_py(gpu.call("pfnIndex", dev_view(gpu, v, H_E, 1), dev_view(gpu, idx, H_L, 1)))
    assert np.array_equal(got, v[1:][idx[1:]])
    got = gpu.to_py(gpu.call("pfnGeq", dev_view(gpu, v, H_E, 1), gpu.scalar(0.25, H_E)))
    want = ora.to_py(ora.call("pfnGeq", ora.vec(v[1:], H_E), ora.scalar(0.25, H_E)))
    assert np.array_equal(got, want)
    gpu.free_inputs()
    ora.free_inputs()


def test_group_sum_tree_order(libs):
    """Per-group f64 sums follow the fixed tile-tree order exactly for every
    segment size class (1, 2, 3-4, ..., 17-32, 33-4096, longer): each equals
    the oracle's restatement of that order over the group's rows, -0.0
    payloads included."""
    gpu, ora = libs
    rng = np.random.default_rng(45)
    sizes = [1, 1, 2, 3, 4, 5, 7, 8, 9, 15, 16, 17, 31, 32, 33, 100, 255, 256, 257, 4095, 4096, 4097, 10_000, 70_000]
    key = np.repeat(np.arange(len(sizes), dtype=np.int64), sizes)
    rng.shuffle(key)
    pay = rng.standard_normal(key.size) * 10.0 ** rng.integers(-8, 8, key.size)
    pay[rng.random(key.size) < 0.01] = -0.0
    pay[np.flatnonzero(key == 0)] = -0.0  # a one-row group holding -0.0
    g = gpu.call("pfnGroup", gpu.vec(key, H_L))
    vals = gpu.call("pfnValues", g)
    sums = gpu.to_py(gpu.call("hgpuGroupSum", gpu.vec(pay, H_E), vals))
    keys = gpu.to_py(gpu.call("pfnKeys", g))
    for gi, first in enumerate(keys):
        rows = np.flatnonzero(key == key[first])
        x = np.ascontiguousarray(pay[rows])
        want = ora.lib.hgoTreeSumF64(x.ctypes.data, x.size)
        assert sums[gi].tobytes() == np.float64(want).tobytes(), (len(rows), sums[gi], want)
    gpu.free_inputs()


@pytest.mark.parametrize("shape", ["two_long", "many_long", "groups_over_4096"])
def test_group_sum_plans(libs, shape):
    """The long groups' chunks run in an interleaved order (planned inside
    @group for 2 to 64 long groups among at most 4096 groups, by the general
    plan for up to 2048 long groups over at least 4M rows) or in group order:
    every shape gives each group the tile tree's sum of its rows, bit for
    bit, and hgpuGroupAggMany agrees with the single calls."""
    from horsepower_gb300 import plans as P
    gpu, ora = libs
    rng = np.random.default_rng(48)
    if shape == "two_long":
        sizes = [9_000, 300_001]
    elif shape == "many_long":
        sizes = list(rng.integers(4_097, 30_000, 100)) + list(rng.integers(1, 300, 200))
    else:  # more than 4096 groups and over 4M rows: the general plan builds the chunk order
        sizes = list(rng.integers(400_000, 600_000, 10)) + list(rng.integers(1, 40, 5_000))
    key = np.repeat(rng.permutation(len(sizes)).astype(np.int64) * 7 - 3, sizes)
    rng.shuffle(key)
    pay = rng.standard_normal(key.size) * 10.0 ** rng.integers(-6, 6, key.size)
    g = gpu.call("pfnGroup", gpu.vec(key, H_L))
    vals = gpu.call("pfnValues", g)
    keys = gpu.to_py(gpu.call("pfnKeys", g))
    sums = gpu.to_py(gpu.call("hgpuGroupSum", gpu.vec(pay, H_E), vals))
    order = np.argsort(key, kind="stable")
    bounds = np.flatnonzero(np.diff(key[order])) + 1
    by_key = {int(key[r[0]]): r for r in np.split(order, bounds)}
    for gi, first in enumerate(keys):
        x = np.ascontiguousarray(pay[by_key[int(key[first])]])
        want = ora.lib.hgoTreeSumF64(x.ctypes.data, x.size)
        assert sums[gi].tobytes() == np.float64(want).tobytes(), (gi, x.size)
    cols = [gpu.vec(rng.uniform(0, 1e5, key.size), H_E) for _ in range(3)]
    pairs = [("pfnSum", cols[0]), ("pfnAvg", cols[1]), ("pfnSum", cols[2]), ("pfnLen", cols[0])]
    many = [gpu.to_py(z) for z in P.group_agg_many(gpu, pairs, vals)]
    single = [gpu.to_py(P.group_agg(gpu, a, x, vals)) for a, x in pairs]
    for a, b in zip(many, single):
        assert a.dtype == b.dtype and a.tobytes() == b.tobytes()
    gpu.free_inputs()


@pytest.mark.parametrize("ops", [["eq", "lt"], ["geq", "eq", "neq"], ["eq", "eq"]])
def test_join_multi_large(libs, ops):
    """Multi-column @join_index at 1M x 3M rows with repeated keys: GPU vs oracle."""
    rng = np.random.default_rng(46)
    nb, npr = 1_000_000, 3_000_000
    cols_b = [rng.integers(0, 400_000, nb).astype(np.int32), rng.integers(0, 60, nb).astype(np.int64),
              np.round(rng.standard_normal(nb), 2)]
    cols_p = [rng.integers(0, 400_000, npr).astype(np.int32), rng.integers(0, 60, npr).astype(np.int32),
              np.round(rng.standard_normal(npr), 2)]
    types_b, types_p = [H_I, H_L, H_E], [H_I, H_I, H_E]
    k = len(ops)
    if ops[0] != "eq":  # put the key column where the first @eq is
        cols_b = [cols_b[1], cols_b[0], cols_b[2]]
        cols_p = [cols_p[1], cols_p[0], cols_p[2]]
        types_b = [types_b[1], types_b[0], types_b[2]]
        types_p = [types_p[1], types_p[0], types_p[2]]
    a, b = both(libs, "pfnJoinIndex", lambda L: (L.list([L.vec(c, t) for c, t in zip(cols_b[:k], types_b[:k])]),
                                                 L.list([L.vec(c, t) for c, t in zip(cols_p[:k], types_p[:k])]),
                                                 L.syms(ops)))
    assert same(a, b) and a[0].size > 0


@pytest.mark.parametrize("typ,lo,hi", [(H_I, 0, 50), (H_L, 1000, 1200), (H_I, 0, 300), (H_I, -5, 40), (H_L, 0, 70000)])
def test_group_narrow_ints(libs, typ, lo, hi):
    """@group on one integer column: narrow non-negative ranges with at most
    256 values take the counting path, others the radix path; both equal the
    oracle's group dict (keys, and every group's rows in order)."""
    rng = np.random.default_rng(hi)
    x = rng.integers(lo, hi, 300_000).astype(np.int32 if typ == H_I else np.int64)
    a, b = both(libs, "pfnGroup", lambda L: (L.vec(x, typ),))
    assert same(a, b)


def index_many(L, cols, idx):
    fn = L.lib.hgpuIndexMany
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong]
    zs = [L.node() for _ in cols]
    rc = fn(L.node_array(zs), L.node_array(cols), C.byref(idx), len(cols))
    return rc, zs


@pytest.mark.parametrize("ityp", [H_L, H_I, 1])
@pytest.mark.parametrize("n", [0, 1, 7, 1_000_003])
def test_index_many_matches_separate_index(libs, ityp, n):
    """hgpuIndexMany (the common index pattern, pattern.cc:558-672) equals one
    pfnIndex per column: ten columns of every element width (two launches of
    up to eight columns), index widths i64/i32/i8, ragged lengths."""
    rng = np.random.default_rng(18)
    nx = 120 if ityp == 1 else 3_000_017
    cols = [(H_B, rng.random(nx) < 0.5), (1, rng.integers(-128, 127, nx).astype(np.int8)),
            (2, rng.integers(-30000, 30000, nx).astype(np.int16)), (H_I, rng.integers(-9, 9, nx).astype(np.int32)),
            (H_L, rng.integers(-2 ** 60, 2 ** 60, nx)), (H_E, rng.standard_normal(nx)),
            (H_C, rng.integers(65, 90, nx).astype(np.int8)), (12, rng.integers(19900101, 19991231, nx).astype(np.int32)),
            (5, rng.standard_normal(nx).astype(np.float32)), (H_L, np.arange(nx, dtype=np.int64))]
    idx = rng.integers(0, nx, n)
    outs = []
    for L in libs:
        xs = [L.vec(a, t) for t, a in cols]
        y = L.vec(idx, ityp)
        rc, zs = index_many(L, xs, y)
        assert rc == 0
        outs.append([L.to_py(z) for z in zs])
        sep = [L.to_py(L.call("pfnIndex", x, y)) for x in xs]
        assert all(same(a, b) for a, b in zip(outs[-1], sep))
        L.free_inputs()
    assert all(same(a, b) for a, b in zip(*outs))


def test_index_many_errors(libs):
    gpu = libs[0]
    rng = np.random.default_rng(19)
    a, b = rng.standard_normal(1000), rng.integers(0, 5, 500).astype(np.int32)
    for bad in (1000, 500, -1):  # outside both, outside the shorter column only, negative
        idx = rng.integers(0, 500, 100_000)
        idx[77_777] = bad
        rc, _ = index_many(gpu, [gpu.vec(a, H_E), gpu.vec(b, H_I)], gpu.vec(idx, H_L))
        assert rc == 3, rc  # E_INDEX
    rc, _ = index_many(gpu, [gpu.vec(a, H_E), gpu.vec(b, H_I)], gpu.vec(rng.random(10), H_E))
    assert rc == 1  # E_DOMAIN: a float index
    # the library is still usable after the errors
    rc, zs = index_many(gpu, [gpu.vec(a, H_E), gpu.vec(b, H_I)], gpu.vec(np.array([3, 499], np.int64), H_L))
    assert rc == 0 and gpu.to_py(zs[0]).tolist() == [a[3], a[499]] and gpu.to_py(zs[1]).tolist() == [b[3], b[499]]
    gpu.free_inputs()


def test_heap_offset_is_a_position(libs):
    """getHeapOffset (h_memory.cc:155-157) reads the arenas' position without
    allocating: repeated reads give the same value, an output moves it
    forward, and setHeapOffset returns both arenas to a value read earlier."""
    gpu = libs[0]
    Lb = gpu.lib
    a = Lb.getHeapOffset()
    assert all(Lb.getHeapOffset() == a for _ in range(100))
    z = gpu.call("pfnPlus", gpu.vec(np.arange(100_000, dtype=np.int64), H_L), gpu.vec(np.ones(100_000, np.int64), H_L))
    lst = gpu.call("pfnGroup", gpu.vec(np.arange(1000, dtype=np.int32) % 7, H_I))  # host nodes too
    b = Lb.getHeapOffset()
    assert b > a and Lb.getHeapOffset() == b
    Lb.setHeapOffset(a)
    assert Lb.getHeapOffset() == a
    z2 = gpu.call("pfnPlus", gpu.vec(np.arange(100_000, dtype=np.int64), H_L), gpu.vec(np.ones(100_000, np.int64), H_L))
    assert z2.g == z.g  # the rewound region is reused
    del lst
    gpu.free_inputs()


QS_CASES = {
    # the reference's quicksort on keys other than i32/i64/char (lib_quicksort_other h_libs.cc:409-442)
    "order_f64_ties": ("pfnOrderBy", lambda r, n: [("vec", np.round(r.standard_normal(n), 1), H_E)], [1]),
    "order_f64_desc": ("pfnOrderBy", lambda r, n: [("vec", np.round(r.standard_normal(n), 2), H_E)], [0]),
    "order_f32": ("pfnOrderBy", lambda r, n: [("vec", np.round(r.standard_normal(n), 1).astype(np.float32), 5)], [1]),
    "order_i8": ("pfnOrderBy", lambda r, n: [("vec", r.integers(-3, 3, n).astype(np.int8), 1)], [1]),
    "order_i16": ("pfnOrderBy", lambda r, n: [("vec", r.integers(-500, 500, n).astype(np.int16), 2)], [0]),
    "order_bool": ("pfnOrderBy", lambda r, n: [("vec", r.random(n) < 0.4, H_B)], [1]),
    "group_f64": ("pfnGroup", lambda r, n: [("vec", np.round(r.standard_normal(n), 1), H_E)], None),
    "group_i16": ("pfnGroup", lambda r, n: [("vec", r.integers(0, 1000, n).astype(np.int16), 2)], None),
    # lib_quicksort_list over lists holding them (h_libs.cc:637-697)
    "group_list_jj": ("pfnGroup", lambda r, n: [("list", [(r.integers(0, 3, n).astype(np.int8), 1),
                                                          (r.integers(0, 2, n).astype(np.int8), 1)])], None),
    "group_list_ei": ("pfnGroup", lambda r, n: [("list", [(np.round(r.standard_normal(n), 0), H_E),
                                                          (r.integers(0, 100, n).astype(np.int32), H_I)])], None),
    "order_list_ei": ("pfnOrderBy", lambda r, n: [("list", [(np.round(r.standard_normal(n), 1), H_E),
                                                            (r.integers(0, 1000, n).astype(np.int32), H_I)])], [0, 1]),
    "order_list_jel": ("pfnOrderBy", lambda r, n: [("list", [(r.integers(0, 4, n).astype(np.int8), 1),
                                                             (np.round(r.standard_normal(n), 1), H_E),
                                                             (r.integers(0, 50, n).astype(np.int64), H_L)])], [1, 0, 1]),
    "order_list_ci": ("pfnOrderBy", lambda r, n: [("list", [(r.integers(65, 91, n).astype(np.int8), H_C),
                                                            (r.integers(0, 300, n).astype(np.int32), H_I)])], [1, 1]),
}


@pytest.mark.parametrize("kind", sorted(QS_CASES))
def test_quicksort_paths_large(libs, kind):
    """The reference's quicksort (and the list sort around it) reproduced
    step for step: the permutation, or the groups with their keys and row
    order, bit-exact against the oracle's restatement at 1.5M rows."""
    fn, mk, dirs = QS_CASES[kind]
    import zlib
    rng = np.random.default_rng(zlib.crc32(kind.encode()))
    spec = mk(rng, 1_500_000)

    def args(L):
        out = []
        for a in spec:
            if a[0] == "vec":
                out.append(L.vec(a[1], a[2]))
            else:
                out.append(L.list([L.vec(v, t) for v, t in a[1]]))
        if dirs is not None:
            out.append(L.vec(np.array(dirs, bool), H_B))
        return tuple(out)
    a, b = both(libs, fn, args)
    assert same(a, b)


def test_quicksort_nan_key_refused(libs):
    """A NaN key sends the reference's quicksort outside its range
    (undefined): the library refuses it with E_NOT_IMPL and stays usable."""
    gpu = libs[0]
    x = np.round(np.random.default_rng(3).standard_normal(5000), 1)
    x[1234] = np.nan
    rc = gpu.rc("pfnOrderBy", gpu.vec(x, H_E), gpu.vec(np.array([1], bool), H_B))
    assert rc == 99
    rc = gpu.rc("pfnGroup", gpu.vec(x, H_E))
    assert rc == 99
    ok = gpu.to_py(gpu.call("pfnOrderBy", gpu.vec(np.nan_to_num(x), H_E), gpu.vec(np.array([1], bool), H_B)))
    assert ok.size == x.size
    gpu.free_inputs()


@pytest.mark.parametrize("shape", ["long_groups", "mixed_sizes", "types"])
def test_group_agg_many_matches_single_calls(libs, shape):
    """hgpuGroupAggMany returns, bit for bit, what one hgpuGroupSum / Avg /
    Min / Max / Len call per column returns: the shared pass over long groups
    (shape long_groups), the per-column path for groups of every size class,
    and non-f64 columns."""
    from horsepower_gb300 import plans as P
    gpu = libs[0]
    rng = np.random.default_rng(47)
    n = 6_000_000
    if shape == "long_groups":
        key = rng.integers(0, 6, n).astype(np.int8)
        g = gpu.call("pfnGroup", gpu.list([gpu.vec(key, H_C), gpu.vec(rng.integers(0, 2, n).astype(np.int8), H_C)]))
    else:
        key = np.minimum(rng.zipf(1.3, n), 100_000).astype(np.int64)
        g = gpu.call("pfnGroup", gpu.vec(key, H_L))
    vals = gpu.call("pfnValues", g)
    cols = [gpu.vec(rng.uniform(0, 1e5, n), H_E) for _ in range(3)]
    if shape == "types":
        cols = [gpu.vec(rng.integers(-9, 9, n).astype(np.int32), H_I), gpu.vec(rng.standard_normal(n).astype(np.float32), 5),
                gpu.vec(rng.uniform(0, 1e5, n), H_E)]
    pairs = [("pfnSum", cols[0]), ("pfnAvg", cols[1]), ("pfnSum", cols[2]), ("pfnLen", cols[0]),
             ("pfnMax", cols[2]), ("pfnAvg", cols[2])]
    many = [gpu.to_py(z) for z in P.group_agg_many(gpu, pairs, vals)]
    single = [gpu.to_py(P.group_agg(gpu, a, x, vals)) for a, x in pairs]
    for a, b in zip(many, single):
        assert a.dtype == b.dtype and a.tobytes() == b.tobytes()
    gpu.free_inputs()
