"""Seeded synthetic tables with the shapes of the benchmark configurations.

The reference quotes TPC-H-shaped queries (6,001,215 rows = SF1 lineitem,
59,986,052 = SF10 lineitem).  Its data generator is not available, so these
seeded tables with the same row counts, types and value distributions stand
in for it:

  filter_table   6,001,215 rows: qty i32 U{1..50}; price f64 =
                 round(qty*U(900,105000)/100, 2); disc f64 = k/100, k U{0..10};
                 shipdate i32 day number U over a 2,526-day range
  join_tables    fact 59,986,052 rows (fk i32 U[0,D), flag/status 1-byte
                 chars in {0,1,2}/{0,1}, qty/price/disc f64 as above) and a
                 dimension of 15,000,000 rows (pk i32 = permutation of 0..D-1,
                 date i32 U over 2,526 days)
  group_table    150,000,000 rows: key i64 ~ Zipf(s=1.1) over 10,000,000 ranks,
                 payload f64 U(0,1e5), sec i32 U[0, 2^20]
"""
import numpy as np

DAYS0 = 8035            # 1992-01-01 as days since 1970-01-01
NDAYS = 2526            # 1992-01-01 .. 1998-12-01
WIN_LO = 8766           # 1994-01-01
WIN_HI = WIN_LO + 365   # 1995-01-01


def _price_disc(rng, qty):
    n = qty.size
    price = np.round(qty.astype(np.float64) * rng.uniform(900.0, 105000.0, n) / 100.0, 2)
    disc = rng.integers(0, 11, n).astype(np.float64) / 100.0
    return price, disc


def filter_table(n=6_001_215, seed=0):
    rng = np.random.default_rng(seed * 1000 + 1)
    qty = rng.integers(1, 51, n).astype(np.int32)
    price, disc = _price_disc(rng, qty)
    shipdate = (DAYS0 + rng.integers(0, NDAYS, n)).astype(np.int32)
    return dict(qty=qty, price=price, disc=disc, shipdate=shipdate)


def join_tables(nfact=59_986_052, ndim=15_000_000, seed=1):
    rng = np.random.default_rng(seed * 1000 + 1)
    pk = rng.permutation(ndim).astype(np.int32)
    date = (DAYS0 + rng.integers(0, NDAYS, ndim)).astype(np.int32)
    fk = rng.integers(0, ndim, nfact).astype(np.int32)
    flag = rng.integers(0, 3, nfact).astype(np.int8)
    status = rng.integers(0, 2, nfact).astype(np.int8)
    qty = rng.integers(1, 51, nfact).astype(np.float64)
    price, disc = _price_disc(rng, qty)
    return dict(pk=pk, date=date), dict(fk=fk, flag=flag, status=status, qty=qty, price=price, disc=disc)


def zipf_cdf(nranks=10_000_000, s=1.1):
    w = np.arange(1, nranks + 1, dtype=np.float64) ** (-s)
    c = np.cumsum(w)
    return c / c[-1]


def group_table(n=150_000_000, nranks=10_000_000, seed=2, chunk=10_000_000):
    rng = np.random.default_rng(seed * 1000 + 1)
    cdf = zipf_cdf(nranks)
    key = np.empty(n, np.int64)
    for i in range(0, n, chunk):
        m = min(chunk, n - i)
        key[i:i + m] = np.searchsorted(cdf, rng.random(m), side="right") + 1
    np.minimum(key, nranks, out=key)
    payload = rng.uniform(0.0, 1e5, n)
    sec = rng.integers(0, 2 ** 20 + 1, n).astype(np.int32)
    return dict(key=key, payload=payload, sec=sec)
