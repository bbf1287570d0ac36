"""The served form (hgpuServerRun) from Python: resident tables, a seeded
request stream with Poisson arrivals, and the loop's latency statistics.

Request mix: 60% filter-aggregates over the lineitem table (random 365-day
shipdate window), 30% join + group-bys (random 365-day dimension date
window), 10% top-1000 orders over a random key range of the order table.
"""
import ctypes as C

import numpy as np

from . import batch as B
from . import data as D
from .abi import V0

FILTER_AGG, JOIN_GROUP, TOPK_ORDER = 0, 1, 2
TOPK = 1000
BATCHED, PLAIN = 0, 1


class Tables(C.Structure):
    _fields_ = [("l_shipdate", C.c_void_p), ("l_qty", C.c_void_p), ("l_disc", C.c_void_p), ("l_price", C.c_void_p),
                ("nline", C.c_longlong),
                ("dim_pk", C.c_void_p), ("dim_date", C.c_void_p), ("ndim", C.c_longlong),
                ("fk", C.c_void_p), ("flag", C.c_void_p), ("status", C.c_void_p), ("qty", C.c_void_p),
                ("price", C.c_void_p), ("disc", C.c_void_p), ("nfact", C.c_longlong),
                ("o_key", C.c_void_p), ("o_sec", C.c_void_p), ("norder", C.c_longlong)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int32), ("lo", C.c_int32), ("hi", C.c_int32), ("klo", C.c_longlong),
                ("khi", C.c_longlong), ("arrival_s", C.c_double)]


class Response(C.Structure):
    _fields_ = [("status", C.c_int32), ("value", C.c_double), ("group", C.POINTER(B.Result)),
                ("rows", C.POINTER(C.c_longlong)), ("nrows", C.c_longlong), ("admit_s", C.c_double),
                ("done_s", C.c_double), ("step", C.c_longlong), ("footprint", C.c_longlong)]


class Stats(C.Structure):
    _fields_ = [("steps", C.c_longlong), ("rejected", C.c_longlong), ("max_step_requests", C.c_longlong),
                ("max_step_bytes", C.c_longlong), ("wall_s", C.c_double), ("qps", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double)]


def _bind(L):
    lib = L.lib
    lib.hgpuServerCreate.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Tables), C.c_longlong, C.c_longlong]
    lib.hgpuServerRun.argtypes = [C.c_void_p, C.POINTER(Request), C.c_longlong, C.POINTER(Response), C.c_int32,
                                  C.POINTER(Stats)]
    lib.hgpuServerFootprint.argtypes = [C.c_void_p, C.POINTER(Request)]
    lib.hgpuServerFootprint.restype = C.c_longlong
    lib.hgpuServerDestroy.argtypes = [C.c_void_p]


def order_table(L, n, seed, nranks=10_000_000, s=1.1):
    """Device-resident (key i64 Zipf(s) over 1..nranks, sec i32) of n rows,
    generated on the device (hgpuSynthOrderTable)."""
    o = V0()
    L.lib.hgpuSynthOrderTable.argtypes = [C.c_ulonglong, C.c_longlong, C.c_longlong, C.c_double, C.c_void_p]
    rc = L.lib.hgpuSynthOrderTable(seed, n, nranks, s, C.byref(o))
    if rc:
        raise RuntimeError(f"hgpuSynthOrderTable: {rc} {L.lib.hgpuLastError().decode()}")
    L._keep.append(o)
    return dict(key=V0.from_address(o.g), sec=V0.from_address(o.g + 32))


def line_table(L, n, seed):
    from .abi import H_E, H_I
    t = D.filter_table(n, seed=seed)
    return dict(shipdate=B.to_device(L, t["shipdate"], H_I), qty=B.to_device(L, t["qty"], H_I),
                disc=B.to_device(L, t["disc"], H_E), price=B.to_device(L, t["price"], H_E))


class Server:
    def __init__(self, L, line, dim, fact, order, budget=0, max_step=0):
        _bind(L)
        self.L = L
        self.tables = Tables(line["shipdate"].g, line["qty"].g, line["disc"].g, line["price"].g, line["qty"].len,
                             dim["pk"].g, dim["date"].g, dim["pk"].len,
                             fact["fk"].g, fact["flag"].g, fact["status"].g, fact["qty"].g, fact["price"].g,
                             fact["disc"].g, fact["fk"].len, order["key"].g, order["sec"].g, order["key"].len)
        self.h = C.c_void_p()
        rc = L.lib.hgpuServerCreate(C.byref(self.h), C.byref(self.tables), budget, max_step)
        if rc:
            raise RuntimeError(f"hgpuServerCreate: {rc} {L.lib.hgpuLastError().decode()}")

    def footprint(self, r):
        return self.L.lib.hgpuServerFootprint(self.h, C.byref(r))

    def run(self, reqs, mode=BATCHED):
        n = len(reqs)
        arr = (Request * max(n, 1))(*reqs)
        out = (Response * max(n, 1))()
        groups = (B.Result * max(n, 1))()
        rows = (C.c_longlong * (TOPK * max(n, 1)))()
        for i in range(n):
            out[i].group = C.pointer(groups[i])
            out[i].rows = C.cast(C.byref(rows, 8 * TOPK * i), C.POINTER(C.c_longlong))
        st = Stats()
        rc = self.L.lib.hgpuServerRun(self.h, arr, n, out, mode, C.byref(st))
        if rc:
            raise RuntimeError(f"hgpuServerRun: {rc} {self.L.lib.hgpuLastError().decode()}")
        res = []
        for i in range(n):
            o = out[i]
            if o.status:
                res.append(("error", o.status))
            elif reqs[i].kind == FILTER_AGG:
                res.append(o.value)
            elif reqs[i].kind == JOIN_GROUP:
                res.append(B.result_rows(groups[i]))
            else:
                res.append(np.ctypeslib.as_array(rows)[TOPK * i:TOPK * i + o.nrows].copy())
        meta = [dict(step=out[i].step, admit_s=out[i].admit_s, done_s=out[i].done_s, footprint=out[i].footprint,
                     status=out[i].status) for i in range(n)]
        return res, st, meta

    def close(self):
        if self.h:
            self.L.lib.hgpuServerDestroy(self.h)
            self.h = C.c_void_p()


def request_stream(n, rate, seed, key_hi=10_000_000, mix=(0.6, 0.3, 0.1), t0=0.0):
    """n requests with Poisson arrivals at `rate` per second."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n) if rate > 0 else np.zeros(n)
    t = t0 + np.cumsum(gaps) - (gaps[0] if n else 0.0)
    kinds = rng.choice(3, n, p=list(mix))
    reqs = []
    for i in range(n):
        lo = int(D.DAYS0 + rng.integers(0, D.NDAYS - 365))
        a = int(rng.integers(1, key_hi))
        b = int(a + rng.integers(1, 200_000))
        reqs.append(Request(int(kinds[i]), lo, lo + 365, a, b, float(t[i])))
    return reqs


def same_result(a, b):
    if isinstance(a, float):
        return isinstance(b, float) and a == b
    if isinstance(a, tuple):
        return isinstance(b, tuple) and len(a) == len(b) and all(
            np.array_equal(x, y) if isinstance(x, np.ndarray) else x == y for x, y in zip(a, b))
    return isinstance(b, np.ndarray) and np.array_equal(a, b)
