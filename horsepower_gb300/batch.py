"""Batched filter-join-aggregate plans (hgpuBatchJoinGroup) from Python.

A plan is the join + group-by query of `plans.join_group` over one pair of
device-resident tables; `run_batch` runs many of them through the library's
batched executor and returns, per plan, the rows of its result in the order
the plain builtins produce them: (flag, status, sum_qty, avg_price, sum_disc,
count) per group, groups ascending by (flag << 8 | status).
"""
import ctypes as C

import numpy as np

from .abi import V0
from . import data as D

MAXG = 256


class Plan(C.Structure):
    _fields_ = [("dim_pk", C.c_void_p), ("dim_date", C.c_void_p), ("ndim", C.c_longlong),
                ("fk", C.c_void_p), ("flag", C.c_void_p), ("status", C.c_void_p),
                ("qty", C.c_void_p), ("price", C.c_void_p), ("disc", C.c_void_p), ("nfact", C.c_longlong),
                ("lo", C.c_int32), ("hi", C.c_int32)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int32), ("ngroups", C.c_longlong),
                ("flag", C.c_int8 * MAXG), ("st", C.c_int8 * MAXG),
                ("sum_qty", C.c_double * MAXG), ("avg_price", C.c_double * MAXG),
                ("sum_disc", C.c_double * MAXG), ("count", C.c_longlong * MAXG)]


def synth_tables(L, seed, nfact, ndim):
    """Device-resident (dim, fact) dicts of V0 nodes from hgpuSynthJoinTables."""
    d, f = V0(), V0()
    L.lib.hgpuSynthJoinTables.argtypes = [C.c_ulonglong, C.c_longlong, C.c_longlong, C.c_void_p, C.c_void_p]
    rc = L.lib.hgpuSynthJoinTables(seed, nfact, ndim, C.byref(d), C.byref(f))
    if rc:
        raise RuntimeError(f"hgpuSynthJoinTables: {rc} {L.lib.hgpuLastError().decode()}")
    L._keep.append((d, f))
    dn = [V0.from_address(d.g + 32 * i) for i in range(2)]
    fn = [V0.from_address(f.g + 32 * i) for i in range(6)]
    return dict(pk=dn[0], date=dn[1]), dict(fk=fn[0], flag=fn[1], status=fn[2], qty=fn[3], price=fn[4], disc=fn[5])


def to_device(L, arr, typ):
    """A device-resident copy of a numpy column (hgpuToDevice)."""
    h = L.vec(arr, typ)
    d = V0()
    rc = L.lib.hgpuToDevice(C.byref(d), C.byref(h))
    if rc:
        raise RuntimeError(f"hgpuToDevice: {rc}")
    L._keep.append(d)
    return d


def device_tables(L, dim, fact):
    """Device copies of host (dim, fact) numpy column dicts."""
    from . import plans as P
    return ({k: to_device(L, v, P.DIM_TYPES[k]) for k, v in dim.items()},
            {k: to_device(L, v, P.FACT_TYPES[k]) for k, v in fact.items()})


def make_plan(dim, fact, lo=D.WIN_LO, hi=D.WIN_HI):
    return Plan(dim["pk"].g, dim["date"].g, dim["pk"].len, fact["fk"].g, fact["flag"].g, fact["status"].g,
                fact["qty"].g, fact["price"].g, fact["disc"].g, fact["fk"].len, lo, hi)


def run_batch(L, plans):
    n = len(plans)
    arr = (Plan * n)(*plans)
    res = (Result * n)()
    L.lib.hgpuBatchJoinGroup.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p]
    rc = L.lib.hgpuBatchJoinGroup(arr, n, res)
    if rc:
        raise RuntimeError(f"hgpuBatchJoinGroup: {rc} {L.lib.hgpuLastError().decode()}")
    return [result_rows(r) for r in res]


def result_rows(r):
    if r.status:
        return ("error", r.status)
    g = r.ngroups
    return (np.array(r.flag[:g], np.int8), np.array(r.st[:g], np.int8), np.array(r.sum_qty[:g]),
            np.array(r.avg_price[:g]), np.array(r.sum_disc[:g]), np.array(r.count[:g], np.int64))


def plain_rows(L, dim, fact):
    """The same plan through the plain builtins (plans.join_group)."""
    from . import plans as P
    out = P.join_group(L, dim, fact)
    v = [L.to_py(o) for o in out]
    return (v[0].astype(np.int8), v[1].astype(np.int8), v[2], v[3], v[4], v[5])


def log_uniform_sizes(n, lo=10_000, hi=20_000_000, seed=3000):
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)
