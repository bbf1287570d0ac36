"""Autotuner knobs (hgpuSetTuning) change speed, never results.

Every setting of each knob must give bit-identical outputs: @join_index in
direct-addressed and hashed mode across tile sizes and load factors, @group
and @order across radix digit widths, and batched plans across tile sizes.
"""
import numpy as np
import pytest

from horsepower_gb300 import autotune as T
from horsepower_gb300 import batch as B
from horsepower_gb300.abi import H_B, H_I, H_L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    import horsepower_gb300
    L = horsepower_gb300.load()
    yield L
    T.apply(L, {"tile_rows": 8, "hash_load": 0.5, "radix_bits": 8, "radix_pass": 2})


def outputs(L, fn):
    z = fn()
    return L.to_py(z)


def same(a, b):
    if isinstance(a, np.ndarray):
        return a.dtype == b.dtype and np.array_equal(a, b)
    if isinstance(a, tuple):
        return all(same(p, q) for p, q in zip(a[1:], b[1:]))
    return len(a) == len(b) and all(same(p, q) for p, q in zip(a, b))


@pytest.mark.parametrize("wide", [False, True])
def test_join_knobs(L, wide):
    rng = np.random.default_rng(21)
    nd, nf = 300_000, 2_000_001
    pk = rng.permutation(nd).astype(np.int64) * (5000 if wide else 1)
    build = pk[rng.random(nd) < 0.3]
    probe = rng.choice(pk, nf) + rng.integers(0, 2, nf) * (7 if wide else nd)
    x, y = L.vec(build.astype(np.int32), H_I), L.vec(probe.astype(np.int32), H_I)
    f = L.sym("eq")
    T.apply(L, {"tile_rows": 8, "hash_load": 0.5})
    ref = outputs(L, lambda: L.call("pfnJoinIndex", x, y, f))
    assert ref[0].size > 0
    for tr in (8, 16, 32):
        for hl in (0.5, 0.65, 0.8):
            for jf in (0, 1):
                T.apply(L, {"tile_rows": tr, "hash_load": hl, "join_filter": jf})
                assert same(outputs(L, lambda: L.call("pfnJoinIndex", x, y, f)), ref), (tr, hl, jf)
    T.apply(L, {"tile_rows": 8, "hash_load": 0.5, "join_filter": 0})


def test_join_filter_in_cluster_shared_memory(L):
    """The join + group-by shape (60M probe keys over a 15M-key dimension,
    2.17M selected): the probe with the presence bitmap in a 16-CTA
    cluster's shared memory returns exactly the L2 probe's pairs."""
    rng = np.random.default_rng(22)
    nd, nf = 15_000_000, 20_000_000
    pk = rng.permutation(nd).astype(np.int32)
    build = pk[rng.random(nd) < 0.1445]
    x, y = L.vec(build, H_I), L.vec(rng.integers(0, nd, nf).astype(np.int32), H_I)
    f = L.sym("eq")
    T.apply(L, {"join_filter": 0})
    ref = outputs(L, lambda: L.call("pfnJoinIndex", x, y, f))
    T.apply(L, {"join_filter": 1})
    got = outputs(L, lambda: L.call("pfnJoinIndex", x, y, f))
    T.apply(L, {"join_filter": 0})
    assert ref[0].size > 2_000_000 and same(got, ref)


def test_radix_knobs(L):
    """@order and @group give the same permutation for every digit width and
    both ways of finding a pass's tile offsets."""
    rng = np.random.default_rng(22)
    n = 1_500_000
    key = np.minimum(rng.zipf(1.1, n), 1_000_000).astype(np.int64)
    sec = rng.integers(0, 2 ** 20 + 1, n).astype(np.int32)
    k, s = L.vec(key, H_L), L.vec(sec, H_I)
    d = L.vec(np.array([1, 1], bool), H_B)
    T.apply(L, {"radix_bits": 8})
    T.apply(L, {"radix_pass": 0})
    ref_o = outputs(L, lambda: L.call("pfnOrderBy", L.list([k, s]), d))
    ref_g = outputs(L, lambda: L.call("pfnGroup", k))
    ref_d = outputs(L, lambda: L.call("pfnOrderBy", s, L.vec(np.array([0], bool), H_B)))
    assert np.array_equal(ref_d, np.argsort(sec, kind="stable")[::-1])  # descending = ascending reversed
    for pm in (0, 1, 2):
        for b in (4, 5, 6, 7, 8):
            T.apply(L, {"radix_bits": b, "radix_pass": pm})
            assert T.current(L)["radix_bits"] == b and T.current(L)["radix_pass"] == pm
            assert same(outputs(L, lambda: L.call("pfnOrderBy", L.list([k, s]), d)), ref_o), (b, pm)
            assert same(outputs(L, lambda: L.call("pfnGroup", k)), ref_g), (b, pm)
            # descending (the last pass writes the permutation in reverse) and a 32-bit key
            assert same(outputs(L, lambda: L.call("pfnOrderBy", s, L.vec(np.array([0], bool), H_B))), ref_d), (b, pm)
    T.apply(L, {"radix_bits": 8, "radix_pass": 2})


def test_batched_tile_rows(L):
    tabs = [B.synth_tables(L, 500 + i, n, max(1, n // 4)) for i, n in enumerate([5000, 70_000, 400_000, 1_300_000])]
    plans = [B.make_plan(d, f) for d, f in tabs]
    T.apply(L, {"tile_rows": 8})
    ref = B.run_batch(L, plans)
    for tr in (16, 32):
        T.apply(L, {"tile_rows": tr})
        got = B.run_batch(L, plans)
        for g, r in zip(got, ref):
            for a, b in zip(g, r):
                assert np.array_equal(a, b)
    T.apply(L, {"tile_rows": 8})


def test_tune_and_clamp(L):
    T.apply(L, {"hash_load": 0.95, "radix_bits": 2, "tile_rows": 100, "l2_fetch": 1000, "radix_pass": 7})
    c = T.current(L)
    assert c == {"tile_rows": 32, "hash_load": 0.8, "radix_bits": 4, "l2_fetch": 128, "join_filter": 0,
                 "radix_pass": 2}
    T.apply(L, {"radix_pass": -3})
    assert T.current(L)["radix_pass"] == 0
    T.apply(L, {"radix_pass": 2})
    T.apply(L, {"l2_fetch": 10})
    assert T.current(L)["l2_fetch"] == 32
    tabs = [B.synth_tables(L, 900 + i, n, n // 4) for i, n in enumerate([20_000, 200_000])]
    plans = [B.make_plan(d, f) for d, f in tabs]
    best, table = T.tune(L, lambda: B.run_batch(L, plans), knobs=("tile_rows",), reps=2,
                         check=lambda out: [tuple(a.tobytes() for a in r) for r in out])
    assert best["tile_rows"] in (8, 16, 32) and set(table["tile_rows"]) == {8, 16, 32}
    assert T.current(L)["tile_rows"] == best["tile_rows"]
