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


# ----------------------------------------------------------------- CSV text
# The reference loads lineitem from '|'-separated text with a trailing '|'
# (backend/load_db.cc:111-129: i32 x4, f64 x4, char x2, date x3, sym x2, str).
LINEITEM_TYPES = [3, 3, 3, 3, 6, 6, 6, 6, 8, 8, 12, 12, 12, 9, 9, 10]
LINEITEM_NAMES = ["l_orderkey", "l_partkey", "l_suppkey", "l_linenumber", "l_quantity", "l_extendedprice",
                  "l_discount", "l_tax", "l_returnflag", "l_linestatus", "l_shipdate", "l_commitdate",
                  "l_receiptdate", "l_shipinstruct", "l_shipmode", "l_comment"]
_INSTRUCT = ["DELIVER IN PERSON", "COLLECT COD", "NONE", "TAKE BACK RETURN"]
_MODES = ["REG AIR", "AIR", "RAIL", "SHIP", "TRUCK", "MAIL", "FOB"]


def _digits(m, col, width, values):
    """Right-aligned decimal digits of non-negative ints, left padding spaces."""
    v = values.astype(np.int64).copy()
    for k in range(width - 1, -1, -1):
        d = (v % 10).astype(np.uint8) + 48
        m[:, col + k] = np.where((v > 0) | (k == width - 1), d, 32)
        v //= 10


def _text(m, col, width, choices, idx):
    """Left-aligned texts from `choices`, right padding spaces."""
    tab = np.full((len(choices), width), 32, np.uint8)
    for i, c in enumerate(choices):
        tab[i, :len(c)] = np.frombuffer(c.encode(), np.uint8)
    m[:, col:col + width] = tab[idx]


def lineitem_csv(rows, seed=7):
    """(text bytes, expected columns) of a lineitem-shaped table in the
    reference's .tbl layout, fields space-padded to fixed widths (the reader
    trims them).  Expected values are what strtod / atoi / the date rule give
    for each field: prices are cents / 100.0, which is the correctly rounded
    double of the two-decimal text."""
    rng = np.random.default_rng(seed)
    orderkey = (np.arange(rows, dtype=np.int64) // 4) * 4 + 1
    partkey = rng.integers(1, 200_001, rows)
    suppkey = rng.integers(1, 10_001, rows)
    linenum = rng.integers(1, 8, rows)
    qty = rng.integers(1, 51, rows)
    cents = qty * rng.integers(90_000, 210_001, rows)  # retail price $900-$2100 per unit
    disc = rng.integers(0, 11, rows)
    tax = rng.integers(0, 9, rows)
    flag = rng.integers(0, 3, rows)
    status = rng.integers(0, 2, rows)
    dates = [(rng.integers(1992, 1999, rows), rng.integers(1, 13, rows), rng.integers(1, 29, rows)) for _ in range(3)]
    ins = rng.integers(0, len(_INSTRUCT), rows)
    mode = rng.integers(0, len(_MODES), rows)
    clen = rng.integers(10, 44, rows)
    widths = [9, 7, 6, 1, 5, 9, 4, 4, 1, 1, 10, 10, 10, 17, 7, 43]
    W = sum(widths) + len(widths) + 1
    m = np.empty((rows, W), np.uint8)
    col = 0

    def sep():
        nonlocal col
        m[:, col] = ord("|")
        col += 1

    for vals, w in [(orderkey, 9), (partkey, 7), (suppkey, 6), (linenum, 1)]:
        _digits(m, col, w, vals)
        col += w
        sep()
    for units, hundredths, w in [(qty, np.zeros(rows, np.int64), 5), (cents // 100, cents % 100, 9),
                                 (np.zeros(rows, np.int64), disc, 4), (np.zeros(rows, np.int64), tax, 4)]:
        _digits(m, col, w - 3, units)
        m[:, col + w - 3] = ord(".")
        m[:, col + w - 2] = (hundredths // 10).astype(np.uint8) + 48
        m[:, col + w - 1] = (hundredths % 10).astype(np.uint8) + 48
        col += w
        sep()
    m[:, col] = np.frombuffer(b"ANR", np.uint8)[flag]
    col += 1
    sep()
    m[:, col] = np.frombuffer(b"OF", np.uint8)[status]
    col += 1
    sep()
    for y, mo, d in dates:
        for k, (v, w) in enumerate([(y, 4), (mo, 2), (d, 2)]):
            for j in range(w - 1, -1, -1):
                m[:, col + j] = (v % 10).astype(np.uint8) + 48
                v = v // 10
            col += w
            if k < 2:
                m[:, col] = ord("-")
                col += 1
        sep()
    _text(m, col, 17, _INSTRUCT, ins)
    col += 17
    sep()
    _text(m, col, 7, _MODES, mode)
    col += 7
    sep()
    letters = rng.integers(97, 123, (rows, 43)).astype(np.uint8)
    letters[rng.random((rows, 43)) < 0.15] = 32
    letters[:, 0] = rng.integers(97, 123, rows)
    pos = np.arange(43)[None, :]
    letters[pos == (clen - 1)[:, None]] = 120  # a letter ends each comment
    letters[pos >= clen[:, None]] = 32
    m[:, col:col + 43] = letters
    col += 43
    sep()
    m[:, col] = ord("\n")
    text = m.tobytes()
    comments = [bytes(r[:n]) for r, n in zip(letters, clen)] if rows <= 2_000_000 else None
    exp = {
        "l_orderkey": orderkey.astype(np.int32), "l_partkey": partkey.astype(np.int32),
        "l_suppkey": suppkey.astype(np.int32), "l_linenumber": linenum.astype(np.int32),
        "l_quantity": qty.astype(np.float64), "l_extendedprice": cents / 100.0,
        "l_discount": disc / 100.0, "l_tax": tax / 100.0,
        "l_returnflag": np.frombuffer(b"ANR", np.uint8)[flag].astype(np.int8),
        "l_linestatus": np.frombuffer(b"OF", np.uint8)[status].astype(np.int8),
        "l_shipinstruct": ins, "l_shipmode": mode, "l_comment": comments,
    }
    for name, (y, mo, d) in zip(["l_shipdate", "l_commitdate", "l_receiptdate"], dates):
        exp[name] = (y * 10000 + mo * 100 + d).astype(np.int32)
    return text, exp
