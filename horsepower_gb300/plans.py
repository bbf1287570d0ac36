"""Builtin call sequences of the benchmark queries, in the interpreter's order.

Each plan is the sequence of `pfn*` calls the HorseIR interpreter makes for
the query (one call per `@builtin`, translator/interpreter.cc:278-294), run
through any library with the builtin C ABI.  The shapes follow the
reference's TPC-H programs: `filter_aggregate` is
tests/hyper/online-hir/q6.hir:9-21; `join_group` is the join + low-cardinality
group-by of q1/q3 (q1.hir:9-60, q3.hir:34-73) with char group columns, which
the interpreter groups with pfnGroupTrie; `group_order` is @group with
per-group aggregates plus a two-column stable @order.
"""
from .abi import H_B, H_C, H_E, H_I, H_L
from . import data as D


def filter_aggregate(L, t, lo=D.WIN_LO, hi=D.WIN_HI):
    """q6: sum(price*disc) over date window AND 0.05<=disc<=0.07 AND qty<24."""
    ship, qty, disc, price = t["shipdate"], t["qty"], t["disc"], t["price"]
    t18 = L.call("pfnGeq", ship, L.scalar(lo, H_I))
    t19 = L.call("pfnLt", ship, L.scalar(hi, H_I))
    t20 = L.call("pfnAnd", t18, t19)
    t21 = L.call("pfnLt", qty, L.scalar(24, H_I))
    t22 = L.call("pfnGeq", disc, L.scalar(0.05, H_E))
    t23 = L.call("pfnLeq", disc, L.scalar(0.07, H_E))
    t24 = L.call("pfnAnd", t22, t23)
    t25 = L.call("pfnAnd", t20, t21)
    t26 = L.call("pfnAnd", t25, t24)
    t32 = L.call("pfnCompress", t26, price)
    t33 = L.call("pfnCompress", t26, disc)
    t43 = L.call("pfnMul", t32, t33)
    return L.call("pfnSum", t43)


_FUSED = {"pfnSum": "hgpuGroupSum", "pfnAvg": "hgpuGroupAvg", "pfnMin": "hgpuGroupMin",
          "pfnMax": "hgpuGroupMax", "pfnLen": "hgpuGroupLen"}


def group_agg(L, agg, x, vals):
    """raze(each(@agg, each_right(@index, x, vals))): the fused entry point when
    the library has it (pattern.cc:63-105), else the interpreter's chain."""
    if hasattr(L.lib, _FUSED[agg]):
        return L.call(_FUSED[agg], x, vals)
    t = L.call("pfnEachRight", x, vals, L.fn_ptr("pfnIndex"))
    e = L.call("pfnEach", t, L.fn_ptr(agg))
    return L.call("pfnRaze", e)


_AGG_CODE = {"pfnSum": 0, "pfnAvg": 1, "pfnMin": 2, "pfnMax": 3, "pfnLen": 4}


def group_agg_many(L, pairs, vals):
    """Several (aggregate, column) pairs over one grouping: hgpuGroupAggMany
    where the library has it (the same bits as one call each), else one
    group_agg per pair."""
    import ctypes as C
    from .abi import BuiltinError
    fn = getattr(L.lib, "hgpuGroupAggMany", None)
    if fn is None or len(pairs) < 2:
        return [group_agg(L, a, x, vals) for a, x in pairs]
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong]
    zs = [L.node() for _ in pairs]
    aggs = (C.c_int32 * len(pairs))(*[_AGG_CODE[a] for a, _ in pairs])
    L._keep.append(aggs)
    rc = fn(L.node_array(zs), L.node_array([x for _, x in pairs]), C.byref(vals), aggs, len(pairs))
    if rc:
        raise BuiltinError("hgpuGroupAggMany", rc, L.lib.hgpuLastError().decode() if L.has_device else "")
    return zs


def index_many(L, cols, idx):
    """@index of several columns by one index vector: the reference's common
    index pattern (pattern.cc:558-672) through hgpuIndexMany where the library
    has it, else one pfnIndex per column."""
    import ctypes as C
    from .abi import BuiltinError
    fn = getattr(L.lib, "hgpuIndexMany", None)
    if fn is None or len(cols) < 2:
        return [L.call("pfnIndex", c, idx) for c in cols]
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong]
    zs = [L.node() for _ in cols]
    rc = fn(L.node_array(zs), L.node_array(cols), C.byref(idx), len(cols))
    if rc:
        detail = L.lib.hgpuLastError().decode() if L.has_device else ""
        raise BuiltinError("hgpuIndexMany", rc, detail)
    return zs


def join_group(L, dim, fact, lo=D.WIN_LO, hi=D.WIN_HI):
    """Filter the dimension on its date, join it to the fact table, group the
    matches on (flag, status) and aggregate sum(qty), avg(price), sum(disc),
    count.  Returns (flag, status, sum_qty, avg_price, sum_disc, count) nodes."""
    d1 = L.call("pfnGeq", dim["date"], L.scalar(lo, H_I))
    d2 = L.call("pfnLt", dim["date"], L.scalar(hi, H_I))
    d3 = L.call("pfnAnd", d1, d2)
    pk2 = L.call("pfnCompress", d3, dim["pk"])
    j = L.call("pfnJoinIndex", pk2, fact["fk"], L.sym("eq"))
    fi = L.call("pfnIndex", j, L.scalar(1, H_L))
    # every use of fi is an @index by it (the common index pattern); the
    # measure columns are gathered in a second call, after the group, so
    # uploads of them still in flight (hgpuToDeviceAsync) overlap the rest
    flag, status = index_many(L, [fact["flag"], fact["status"]], fi)
    g = L.call("pfnGroup", L.list([flag, status]))
    keys = L.call("pfnKeys", g)
    vals = L.call("pfnValues", g)
    qty, price, disc = index_many(L, [fact["qty"], fact["price"], fact["disc"]], fi)
    out_flag = L.call("pfnIndex", flag, keys)
    out_status = L.call("pfnIndex", status, keys)
    sum_qty, avg_price, sum_disc, count = group_agg_many(
        L, [("pfnSum", qty), ("pfnAvg", price), ("pfnSum", disc), ("pfnLen", qty)], vals)
    return out_flag, out_status, sum_qty, avg_price, sum_disc, count


_QUERIES = {}


def compiled_queries(L):
    """libhgpu_queries.so (the queries compiled to C, built by build.py), bound
    to the already loaded libhgpu, or None when it is absent."""
    import ctypes as C
    import os
    if id(L) in _QUERIES:
        return _QUERIES[id(L)]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libhgpu_queries.so")
    q = None
    if getattr(L, "has_device", False) and os.path.exists(path):
        q = C.CDLL(path)
        q.hgpuQueryJoinGroup.restype = C.c_int32
        q.hgpuQueryJoinGroup.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
    _QUERIES[id(L)] = q
    return q


def join_group_compiled(L, dim, fact, lo=D.WIN_LO, hi=D.WIN_HI):
    """join_group as the compiled C query (queries/join_group.c): the same
    builtin calls, issued from C instead of Python."""
    from .abi import BuiltinError
    q = compiled_queries(L)
    ins = [dim["date"], dim["pk"], fact["fk"], fact["flag"], fact["status"], fact["qty"], fact["price"], fact["disc"]]
    outs = [L.node() for _ in range(6)]
    rc = q.hgpuQueryJoinGroup(L.node_array(ins), lo, hi, L.node_array(outs))
    if rc:
        raise BuiltinError("hgpuQueryJoinGroup", rc, L.lib.hgpuLastError().decode())
    return tuple(outs)


def group_order(L, t):
    """@group(key) with per-group sum(payload) and count, and the stable
    ascending @order of (key, sec).  Returns (keys, sums, counts, order)."""
    g = L.call("pfnGroup", t["key"])
    keys = L.call("pfnKeys", g)
    vals = L.call("pfnValues", g)
    sums = group_agg(L, "pfnSum", t["payload"], vals)
    counts = group_agg(L, "pfnLen", t["payload"], vals)
    order = L.call("pfnOrderBy", L.list([t["key"], t["sec"]]), L.vec(__import__("numpy").array([1, 1], bool), H_B))
    return keys, sums, counts, order


def host_nodes(L, cols, types):
    """Host vector nodes for a dict of numpy columns."""
    return {k: L.vec(v, types[k]) for k, v in cols.items()}


FILTER_TYPES = dict(qty=H_I, price=H_E, disc=H_E, shipdate=H_I)
DIM_TYPES = dict(pk=H_I, date=H_I)
FACT_TYPES = dict(fk=H_I, flag=H_C, status=H_C, qty=H_E, price=H_E, disc=H_E)
GROUP_TYPES = dict(key=H_L, payload=H_E, sec=H_I)


# The q6 chain as one fused program (autofusion.cc:807-812: a masked
# reduction `if(cond) c += price*disc`).  Inputs: x0 shipdate, x1 qty,
# x2 disc, x3 price.
Q6_CHAIN = ("(sum (mul x3 x2) (and (geq x0 {lo}:i32) (lt x0 {hi}:i32) (lt x1 24:i32) "
            "(geq x2 0.05:f64) (leq x2 0.07:f64)))")


class Chain:
    """A fused chain compiled once by libhgpu (hgpuChainCreate)."""

    def __init__(self, L, program):
        import ctypes as C
        self.L = L
        self.h = C.c_void_p()
        L.lib.hgpuChainCreate.argtypes = [C.c_void_p, C.c_char_p]
        L.lib.hgpuChainRun.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.lib.hgpuChainRunMany.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        rc = L.lib.hgpuChainCreate(C.byref(self.h), program.encode())
        if rc:
            raise RuntimeError(f"hgpuChainCreate: {rc} {L.lib.hgpuLastError().decode()}")

    def run(self, inputs):
        import ctypes as C
        from .abi import V0, BuiltinError
        arr = (C.POINTER(V0) * len(inputs))(*[C.pointer(v) for v in inputs])
        z = self.L.node()
        rc = self.L.lib.hgpuChainRun(self.h, C.byref(z), arr)
        if rc:
            raise BuiltinError("hgpuChainRun", rc, self.L.lib.hgpuLastError().decode())
        return z

    def run_many(self, inputs, nout):
        """A chain with several outputs ((compress M E1 E2 ...), (map E1 E2 ...))."""
        import ctypes as C
        from .abi import V0, BuiltinError
        arr = (C.POINTER(V0) * len(inputs))(*[C.pointer(v) for v in inputs])
        zs = [self.L.node() for _ in range(nout)]
        zarr = (C.POINTER(V0) * nout)(*[C.pointer(z) for z in zs])
        rc = self.L.lib.hgpuChainRunMany(self.h, zarr, arr)
        if rc:
            raise BuiltinError("hgpuChainRunMany", rc, self.L.lib.hgpuLastError().decode())
        return zs


def filter_aggregate_fused(L, t, chain=None, lo=D.WIN_LO, hi=D.WIN_HI):
    chain = chain or Chain(L, Q6_CHAIN.format(lo=lo, hi=hi))
    return chain.run([t["shipdate"], t["qty"], t["disc"], t["price"]])
