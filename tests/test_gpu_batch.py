"""Batched join + group-by plans (hgpuBatchJoinGroup) against the same plans
run one at a time through the builtins.

Bar: bit-exact, f64 sums and averages included: the batched kernels keep
each plan's matched rows in fact-row order and reduce every group with the
same fixed-order tile tree as hgpuGroupSum.  Plans outside the batched
kernels' scope (repeated dimension keys, a key range too wide for a presence
bitmap, a compressed key column longer than the fact table) must come back
identical too, through the per-plan builtin path.
"""
import ctypes as C
import os

import numpy as np
import pytest

from horsepower_gb300 import batch as B
from horsepower_gb300 import data as D

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    import horsepower_gb300
    L = horsepower_gb300.load()
    L.lib.getHeapOffset.restype = C.c_longlong
    L.lib.setHeapOffset.argtypes = [C.c_longlong]
    return L


def identical(a, b):
    assert not isinstance(a[0], str) and not isinstance(b[0], str), (a, b)
    for x, y in zip(a, b):
        assert x.dtype == y.dtype and x.shape == y.shape, (x, y)
        assert np.array_equal(x, y), (x, y)


def plain(L, dim, fact, lo=D.WIN_LO, hi=D.WIN_HI):
    from horsepower_gb300 import plans as P
    mark = L.lib.getHeapOffset()
    out = P.join_group(L, dim, fact, lo, hi)
    v = [L.to_py(o) for o in out]
    L.lib.setHeapOffset(mark)
    return (v[0].astype(np.int8), v[1].astype(np.int8), v[2], v[3], v[4], v[5].astype(np.int64))


def test_synth_tables(L):
    """The generator is a pure function of the seed; pk is a permutation."""
    n, nd = 300_000, 75_000
    d1, f1 = B.synth_tables(L, 7, n, nd)
    d2, f2 = B.synth_tables(L, 7, n, nd)
    d3, f3 = B.synth_tables(L, 8, n, nd)
    for k in d1:
        assert np.array_equal(L.to_py(d1[k]), L.to_py(d2[k]))
    for k in f1:
        assert np.array_equal(L.to_py(f1[k]), L.to_py(f2[k]))
    assert not np.array_equal(L.to_py(f1["fk"]), L.to_py(f3["fk"]))
    pk = L.to_py(d1["pk"])
    assert np.array_equal(np.sort(pk), np.arange(nd, dtype=np.int32))
    date = L.to_py(d1["date"])
    assert date.min() >= D.DAYS0 and date.max() <= D.DAYS0 + 2525
    fk, flag, st = L.to_py(f1["fk"]), L.to_py(f1["flag"]), L.to_py(f1["status"])
    assert fk.min() >= 0 and fk.max() < nd
    assert set(np.unique(flag)) == {0, 1, 2} and set(np.unique(st)) == {0, 1}
    qty, price, disc = L.to_py(f1["qty"]), L.to_py(f1["price"]), L.to_py(f1["disc"])
    assert qty.min() >= 1 and qty.max() <= 50 and np.all(qty == np.round(qty))
    assert np.all(price >= 9.0 * qty - 1e-9) and np.all(price <= 1050.0 * qty + 1e-9)
    assert set(np.round(np.unique(disc) * 100).astype(int)) <= set(range(11))


def test_batch_equals_builtins(L):
    """Plans of every size class, tile-boundary sizes included, in one batch."""
    sizes = [1, 9, 10, 100, 4095, 4096, 4097, 8193, 50_000, 1_000_000, 2_500_000]
    sizes += list(B.log_uniform_sizes(13, 10_000, 600_000, seed=3000))
    tabs, plans = [], []
    for i, n in enumerate(sizes):
        dim, fact = B.synth_tables(L, 3000 + i, int(n), max(1, int(n) // 4))
        tabs.append((dim, fact))
        plans.append(B.make_plan(dim, fact))
    got = B.run_batch(L, plans)
    for (dim, fact), g in zip(tabs, got):
        identical(g, plain(L, dim, fact))


def test_batch_windows(L):
    """An empty window (no matches), a window holding every dimension row,
    and the same tables twice in one batch."""
    dim, fact = B.synth_tables(L, 41, 200_000, 50_000)
    plans = [B.make_plan(dim, fact, 9000, 9000), B.make_plan(dim, fact, 0, 1 << 30),
             B.make_plan(dim, fact), B.make_plan(dim, fact)]
    got = B.run_batch(L, plans)
    assert got[0][0].size == 0
    identical(got[1], plain(L, dim, fact, 0, 1 << 30))
    identical(got[2], plain(L, dim, fact))
    identical(got[3], got[2])


def test_batch_builtin_path(L):
    """Plans outside the batched kernels' scope, mixed with plans inside it."""
    rng = np.random.default_rng(9)
    n, nd = 120_000, 30_000
    fact = dict(fk=rng.integers(0, nd, n).astype(np.int32), flag=rng.integers(0, 3, n).astype(np.int8),
                status=rng.integers(0, 2, n).astype(np.int8), qty=rng.integers(1, 51, n).astype(np.float64),
                price=np.round(rng.uniform(900, 105000, n)) / 100, disc=rng.integers(0, 11, n) / 100)
    date = (8035 + rng.integers(0, 2526, nd)).astype(np.int32)
    dup_pk = rng.integers(0, nd // 2, nd).astype(np.int32)                # repeated keys
    wide_pk = (rng.permutation(nd).astype(np.int64) * 5000).astype(np.int32)  # range ~ 5000 x nd
    cases = [dict(pk=dup_pk, date=date), dict(pk=wide_pk, date=date)]
    devs = [B.device_tables(L, d, fact) for d in cases]
    # a compressed key column longer than the fact table
    dl, fl = B.synth_tables(L, 77, 5_000, 60_000)
    ok_d, ok_f = B.synth_tables(L, 78, 100_000, 25_000)
    plans = [B.make_plan(*devs[0]), B.make_plan(ok_d, ok_f), B.make_plan(*devs[1]),
             B.make_plan(dl, fl, 0, 1 << 30)]
    got = B.run_batch(L, plans)
    identical(got[0], plain(L, *devs[0]))
    identical(got[1], plain(L, ok_d, ok_f))
    identical(got[2], plain(L, *devs[1]))
    identical(got[3], plain(L, dl, fl, 0, 1 << 30))


def test_batch_vs_oracle(L):
    """One small plan against the oracle port (f64 within 1e-12 relative)."""
    import subprocess
    from horsepower_gb300.abi import Builtins
    from horsepower_gb300 import plans as P
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    ora = Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")
    dim, fact = B.synth_tables(L, 5, 400_000, 100_000)
    got = B.run_batch(L, [B.make_plan(dim, fact)])[0]
    hd = {k: L.to_py(v) for k, v in dim.items()}
    hf = {k: L.to_py(v) for k, v in fact.items()}
    r = P.join_group(ora, P.host_nodes(ora, hd, P.DIM_TYPES), P.host_nodes(ora, hf, P.FACT_TYPES))
    want = [ora.to_py(v) for v in r]
    assert np.array_equal(got[0], want[0].astype(np.int8)) and np.array_equal(got[1], want[1].astype(np.int8))
    assert np.array_equal(got[5], want[5])
    for k in (2, 3, 4):
        assert np.allclose(got[k], want[k], rtol=1e-12, atol=0)


def test_shared_tables(L):
    """Plans over identical tables take the shared probe; its results equal
    each plan's builtins, including the cases it must hand back to them (a
    repeated key, a compressed key column longer than the fact table)."""
    dim, fact = B.synth_tables(L, 61, 300_000, 75_000)
    wins = [(D.WIN_LO, D.WIN_HI), (D.DAYS0, D.DAYS0 + 30), (9000, 9000), (0, 1 << 30), (D.WIN_LO, D.WIN_HI)]
    got = B.run_batch(L, [B.make_plan(dim, fact, lo, hi) for lo, hi in wins])
    for (lo, hi), g in zip(wins, got):
        identical(g, plain(L, dim, fact, lo, hi))
    identical(got[0], got[4])
    rng = np.random.default_rng(62)
    n, nd = 50_000, 20_000
    f2 = dict(fk=rng.integers(0, nd, n).astype(np.int32), flag=rng.integers(0, 3, n).astype(np.int8),
              status=rng.integers(0, 2, n).astype(np.int8), qty=rng.integers(1, 51, n).astype(np.float64),
              price=np.round(rng.uniform(900, 105000, n)) / 100, disc=rng.integers(0, 11, n) / 100)
    d2 = dict(pk=rng.integers(0, nd // 2, nd).astype(np.int32), date=(8035 + rng.integers(0, 2526, nd)).astype(np.int32))
    dd, ff = B.device_tables(L, d2, f2)               # repeated keys
    ds, fs = B.synth_tables(L, 63, 4_000, 40_000)     # dimension longer than the fact table
    plans = [B.make_plan(dd, ff), B.make_plan(dd, ff, D.DAYS0, D.DAYS0 + 900),
             B.make_plan(ds, fs, 0, 1 << 30), B.make_plan(ds, fs, D.WIN_LO, D.WIN_LO + 60)]
    got = B.run_batch(L, plans)
    identical(got[0], plain(L, dd, ff))
    identical(got[1], plain(L, dd, ff, D.DAYS0, D.DAYS0 + 900))
    identical(got[2], plain(L, ds, fs, 0, 1 << 30))
    identical(got[3], plain(L, ds, fs, D.WIN_LO, D.WIN_LO + 60))
