"""High-cardinality group-by and stable order at their full size, against the
oracle.

The workload: 150,000,000 rows of i64 keys Zipf(1.1) over 10,000,000 ranks
(about 8.6M distinct keys occur), an i32 secondary column uniform over
[0, 2^20] (both from the device generator the benchmark uses, seed 2) and an
f64 payload uniform over [0, 1e5).  Checked:

* @group(key): the group keys, the concatenated row lists (@raze of the
  values) and the group lengths are bit-exact against the oracle's
  restatement of lib_group_by_normal_long (h_libs.cc:1369-1403);
* per-group sums (hgpuGroupSum) are bit-exact against the oracle's
  restatement of the library's fixed tile-tree order over each group's rows,
  and within 1e-12 relative of the oracle's per-group pfnSum (the
  reference's OpenMP order, h_primitive.cc:764-786);
* @order((key, sec), (1, 1)): the permutation is bit-exact against the
  oracle's lib_quicksort_list (h_libs.cc:637-697: merge sort on key, then on
  sec within each run of equal keys).

The oracle's sorts take about a minute at this size on the host cores.
"""
import ctypes as C
import os
import time

import numpy as np
import pytest

from horsepower_gb300.abi import Builtins, H_B, H_E, H_I, H_L

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 150_000_000
RTOL = 1e-12


@pytest.fixture(scope="module")
def c2():
    import subprocess
    import horsepower_gb300
    from horsepower_gb300 import serve as S
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    ora = Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")
    ora.lib.hgoSegTreeSumF64.restype = None
    ora.lib.hgoSegTreeSumF64.argtypes = [C.c_void_p] * 3 + [C.c_longlong, C.c_longlong, C.c_void_p]
    gpu = horsepower_gb300.load()
    o = S.order_table(gpu, N, seed=2)
    key, sec = gpu.to_py(o["key"]), gpu.to_py(o["sec"])
    pay = np.random.default_rng(2002).uniform(0.0, 1e5, N)
    yield gpu, ora, o, key, sec, pay
    gpu.free_inputs()
    ora.free_inputs()


def _log(msg, t0):
    print(f"{msg}: {time.perf_counter() - t0:.1f} s", flush=True)


def test_c2_shape(c2):
    _, _, _, key, sec, _ = c2
    assert key.dtype == np.int64 and key.size == N and sec.dtype == np.int32 and sec.size == N
    assert key.min() >= 1 and key.max() <= 10_000_000 and sec.min() >= 0 and sec.max() <= 2 ** 20
    assert np.unique(key).size > 5_000_000  # high cardinality


def test_c2_group_full(c2):
    gpu, ora, o, key, _, pay = c2
    t0 = time.perf_counter()
    g = gpu.call("pfnGroup", o["key"])
    gv = gpu.call("pfnValues", g)
    gkeys = gpu.to_py(gpu.call("pfnKeys", g))
    grows = gpu.to_py(gpu.call("pfnRaze", gv))
    glens = gpu.to_py(gpu.call("hgpuGroupLen", gpu.vec(pay, H_E), gv))
    gsums = gpu.to_py(gpu.call("hgpuGroupSum", gpu.vec(pay, H_E), gv))
    _log("gpu group + sums", t0)
    t0 = time.perf_counter()
    og = ora.call("pfnGroup", ora.vec(key, H_L))
    ov = ora.call("pfnValues", og)
    okeys = ora.to_py(ora.call("pfnKeys", og))
    orows = ora.to_py(ora.call("pfnRaze", ov))
    olens = ora.to_py(ora.call("hgpuGroupLen", ora.vec(pay, H_E), ov))
    _log("oracle group", t0)
    assert gkeys.dtype == okeys.dtype and np.array_equal(gkeys, okeys)
    assert np.array_equal(glens, olens)
    assert np.array_equal(grows, orows)
    # per-group sums: the fixed tile-tree order exactly, over the (now known equal) row lists
    starts = np.zeros(len(glens), np.int64)
    np.cumsum(glens[:-1], out=starts[1:])
    want = np.empty(len(glens))
    t0 = time.perf_counter()
    ora.lib.hgoSegTreeSumF64(pay.ctypes.data, orows.ctypes.data, starts.ctypes.data, len(glens), N, want.ctypes.data)
    _log("oracle tree sums", t0)
    assert gsums.tobytes() == want.tobytes()
    # and the reference's own per-group sums (pfnSum, OpenMP order) within the tolerance
    t0 = time.perf_counter()
    osums = ora.to_py(ora.call("hgpuGroupSum", ora.vec(pay, H_E), ov))
    _log("oracle pfnSum per group", t0)
    assert np.allclose(gsums, osums, rtol=RTOL, atol=0)


def test_c2_order_full(c2):
    gpu, ora, o, key, sec, _ = c2
    dirs = np.array([1, 1], bool)
    t0 = time.perf_counter()
    gp = gpu.to_py(gpu.call("pfnOrderBy", gpu.list([o["key"], o["sec"]]), gpu.vec(dirs, H_B)))
    _log("gpu order", t0)
    t0 = time.perf_counter()
    op = ora.to_py(ora.call("pfnOrderBy", ora.list([ora.vec(key, H_L), ora.vec(sec, H_I)]), ora.vec(dirs, H_B)))
    _log("oracle order", t0)
    assert gp.dtype == np.int64 and op.dtype == np.int64
    assert np.array_equal(gp, op)
