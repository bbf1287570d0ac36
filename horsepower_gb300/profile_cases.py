"""Single-builtin workloads for kernel profiling (ncu) and micro-benchmarks.

    python -m horsepower_gb300.profile_cases join      # @join_index, 2.17M build x 60M probe
    python -m horsepower_gb300.profile_cases compress  # @compress f64, 6M rows, 1.8% selected
    python -m horsepower_gb300.profile_cases group     # @group on two 1-byte columns, 8.67M rows
    python -m horsepower_gb300.profile_cases order     # @order (i64 key, i32 sec), N rows
    python -m horsepower_gb300.profile_cases groupkey  # @group on i64 Zipf keys, 150M rows
    python -m horsepower_gb300.profile_cases gather    # @index f64 by ascending row ids
    python -m horsepower_gb300.profile_cases sum       # @sum then @max of f64, N rows
    python -m horsepower_gb300.profile_cases q6        # fused q6 chain, 6M rows
    python -m horsepower_gb300.profile_cases shared    # 16 batched join plans over one pair of tables
    python -m horsepower_gb300.profile_cases csv       # readCSV of a lineitem-shaped .tbl, N rows
    ... --tune tile_rows=32 --tune hash_load=0.7       # autotuner knobs

Inputs are seeded, uploaded once, and each case runs --reps times on
device-resident data, printing the CUDA-event time per call.
"""
import argparse
import ctypes as C

import numpy as np

from . import load
from . import data as D
from .abi import H_B, H_C, H_E, H_I, H_L, V0


def dev(L, arr, typ):
    h = L.vec(arr, typ)
    d = V0()
    assert L.lib.hgpuToDevice(C.byref(d), C.byref(h)) == 0
    L._keep.append(d)
    return d


def timed(L, fn, reps):
    L.lib.hgpuTimerStop.restype = C.c_double
    L.lib.getHeapOffset.restype = C.c_longlong
    out = []
    for _ in range(reps):
        mark = L.lib.getHeapOffset()
        L.lib.hgpuSync()
        L.lib.hgpuTimerStart()
        fn()
        out.append(L.lib.hgpuTimerStop())
        L.lib.setHeapOffset(C.c_longlong(mark))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["join", "compress", "group", "groupkey", "order", "gather", "sum", "q6", "shared", "csv"])
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--rows", type=int, default=0)
    ap.add_argument("--tune", action="append", default=[], help="knob=value (autotuner knobs)")
    a = ap.parse_args()
    L = load()
    if a.tune:
        from . import autotune
        autotune.apply(L, {kv.split("=")[0]: float(kv.split("=")[1]) for kv in a.tune})
    rng = np.random.default_rng(5)
    if a.case == "join":
        F = a.rows or 59_986_052
        D_ = 15_000_000
        pk = rng.permutation(D_).astype(np.int32)
        keep = (rng.integers(0, D.NDAYS, D_) < 365)
        x = dev(L, pk[keep], H_I)
        y = dev(L, rng.integers(0, D_, F).astype(np.int32), H_I)
        f = L.sym("eq")
        t = timed(L, lambda: L.call("pfnJoinIndex", x, y, f), a.reps)
    elif a.case == "compress":
        n = a.rows or 6_001_215
        m = dev(L, rng.random(n) < 0.018, H_B)
        v = dev(L, rng.standard_normal(n), H_E)
        t = timed(L, lambda: L.call("pfnCompress", m, v), a.reps)
    elif a.case == "group":
        n = a.rows or 8_662_796
        f = dev(L, rng.integers(0, 3, n).astype(np.int8), H_C)
        s = dev(L, rng.integers(0, 2, n).astype(np.int8), H_C)
        lst = L.list([f, s])
        t = timed(L, lambda: L.call("pfnGroup", lst), a.reps)
    elif a.case == "groupkey":
        from . import serve as S
        o = S.order_table(L, a.rows or 150_000_000, seed=2)
        t = timed(L, lambda: L.call("pfnGroup", o["key"]), a.reps)
    elif a.case == "order":
        n = a.rows or 20_000_000
        key = dev(L, np.minimum(rng.zipf(1.1, n), 10_000_000).astype(np.int64), H_L)
        sec = dev(L, rng.integers(0, 2 ** 20 + 1, n).astype(np.int32), H_I)
        lst = L.list([key, sec])
        d = L.vec(np.array([1, 1], bool), H_B)
        t = timed(L, lambda: L.call("pfnOrderBy", lst, d), a.reps)
    elif a.case == "gather":
        n = a.rows or 59_986_052
        x = dev(L, rng.standard_normal(n), H_E)
        idx = dev(L, np.flatnonzero(rng.random(n) < 0.1445).astype(np.int64), H_L)
        t = timed(L, lambda: L.call("pfnIndex", x, idx), a.reps)
    elif a.case == "sum":
        n = a.rows or 60_000_000
        x = dev(L, rng.uniform(0, 1e5, n), H_E)
        t = timed(L, lambda: (L.call("pfnSum", x), L.call("pfnMax", x)), a.reps)
    elif a.case == "shared":
        from . import batch as B
        n = a.rows or 59_986_052
        dim, fact = B.synth_tables(L, 1, n, n // 4)
        plans = [B.make_plan(dim, fact, D.DAYS0 + 100 * k, D.DAYS0 + 100 * k + 365) for k in range(16)]
        t = timed(L, lambda: B.run_batch(L, plans), a.reps)
    elif a.case == "csv":
        import os
        import tempfile
        text, _ = D.lineitem_csv(a.rows or 1_000_000, seed=9)
        fd, path = tempfile.mkstemp(suffix=".tbl")
        os.write(fd, text)
        os.close(fd)
        ty = (C.c_longlong * 16)(*D.LINEITEM_TYPES)
        sy = (C.c_longlong * 16)(*[L.lib.getSymbol(n.encode()) for n in D.LINEITEM_NAMES])
        L.lib.hgpuReadCSV.argtypes = [C.c_void_p, C.c_char_p, C.c_longlong, C.c_void_p, C.c_void_p]

        def run():
            z = V0()
            assert L.lib.hgpuReadCSV(C.addressof(z), path.encode(), 16, ty, sy) == 0
        t = timed(L, run, a.reps)
        os.remove(path)
    else:
        from . import plans as P
        tb = D.filter_table(a.rows or 6_001_215)
        nodes = {k: dev(L, v, P.FILTER_TYPES[k]) for k, v in tb.items()}
        ch = P.Chain(L, P.Q6_CHAIN.format(lo=D.WIN_LO, hi=D.WIN_HI))
        t = timed(L, lambda: ch.run([nodes["shipdate"], nodes["qty"], nodes["disc"], nodes["price"]]), a.reps)
    print(f"{a.case}: ms per call {[round(v, 4) for v in t]}")


if __name__ == "__main__":
    main()
