"""The served form (hgpuServerRun): continuous batching over resident tables.

* every result is bit-identical alone (a stream of one request) and in a mix
  of concurrently admitted requests;
* the served results equal the plain one-request-at-a-time builtin path:
  join + group-by and top-k bit-exact, filter-aggregates within 1e-12
  relative (the shared scan sums the full row range in the fused chain's
  order, bit-identical to hgpuChainRun, while @compress then @sum sums the
  compacted rows);
* admission never lets a step's footprint exceed the budget, and a request
  larger than the whole budget is refused with E_ADMISSION;
* small cases agree with the oracle port.
"""
import ctypes as C
import os

import numpy as np
import pytest

from horsepower_gb300 import batch as B
from horsepower_gb300 import data as D
from horsepower_gb300 import serve as S

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
E_ADMISSION = 104


@pytest.fixture(scope="module")
def env():
    import horsepower_gb300
    L = horsepower_gb300.load()
    line = S.line_table(L, 600_000, seed=31)
    dim, fact = B.synth_tables(L, 32, 600_000, 150_000)
    order = S.order_table(L, 1_500_000, seed=33, nranks=100_000)
    srv = S.Server(L, line, dim, fact, order)
    yield L, srv, (line, dim, fact, order)
    srv.close()


def stream(n, seed, rate=0.0):
    return S.request_stream(n, rate, seed, key_hi=100_000)


def test_alone_equals_mix(env):
    L, srv, _ = env
    reqs = stream(48, seed=1)
    mix, st, meta = srv.run(reqs)
    assert st.max_step_requests > 1 and st.rejected == 0
    kinds = {r.kind for r in reqs}
    assert kinds == {0, 1, 2}
    for r, got in zip(reqs, mix):
        alone, _, _ = srv.run([S.Request(r.kind, r.lo, r.hi, r.klo, r.khi, 0.0)])
        assert S.same_result(got, alone[0]), (r.kind, got, alone[0])


def test_served_equals_plain(env):
    L, srv, _ = env
    reqs = stream(30, seed=2)
    served, _, _ = srv.run(reqs, S.BATCHED)
    plain, st, meta = srv.run(reqs, S.PLAIN)
    assert st.max_step_requests == 1 and st.steps == len(reqs)
    for r, a, b in zip(reqs, served, plain):
        if r.kind == S.FILTER_AGG:
            assert abs(a - b) <= 1e-12 * abs(b), (a, b)
        else:
            assert S.same_result(a, b), (r.kind, a, b)


def test_filter_agg_equals_fused_chain(env):
    from horsepower_gb300 import plans as P
    L, srv, (line, _, _, _) = env
    reqs = [S.Request(S.FILTER_AGG, lo, lo + 365, 0, 0, 0.0) for lo in (D.WIN_LO, D.DAYS0, D.DAYS0 + 1000)]
    served, _, _ = srv.run(reqs)
    for r, v in zip(reqs, served):
        ch = P.Chain(L, P.Q6_CHAIN.format(lo=r.lo, hi=r.hi))
        f = L.to_py(ch.run([line["shipdate"], line["qty"], line["disc"], line["price"]]))[0]
        assert v == f, (v, f)


def test_admission_budget(env):
    import horsepower_gb300
    L, _, (line, dim, fact, order) = env
    probe = S.Server(L, line, dim, fact, order)
    reqs = stream(24, seed=3)
    fps = [probe.footprint(r) for r in reqs]
    probe.close()
    budget = 2 * max(fps[i] for i, r in enumerate(reqs) if r.kind == S.JOIN_GROUP)
    srv = S.Server(L, line, dim, fact, order, budget=budget)
    ref, _, _ = env[1].run(reqs)
    got, st, meta = srv.run(reqs)
    assert st.rejected == 0 and st.max_step_bytes <= budget and st.steps > 1
    for a, b in zip(got, ref):
        assert S.same_result(a, b)
    # a request that can never fit is refused; the others still run
    small = S.Server(L, line, dim, fact, order, budget=min(fps) + 1)
    got, st, meta = small.run(reqs)
    for r, g, m, fp in zip(reqs, got, meta, fps):
        if fp > min(fps) + 1:
            assert g == ("error", E_ADMISSION) and m["status"] == E_ADMISSION
        else:
            assert not isinstance(g, tuple) or g[0] != "error"
    assert st.rejected == sum(fp > min(fps) + 1 for fp in fps)
    srv.close()
    small.close()


def test_continuous_batching(env):
    """Requests arriving while a step runs join a later step."""
    L, srv, _ = env
    reqs = stream(200, seed=4, rate=4000.0)
    got, st, meta = srv.run(reqs)
    assert st.rejected == 0 and st.steps < len(reqs) and st.max_step_requests > 1
    for r, m in zip(reqs, meta):
        assert m["admit_s"] >= r.arrival_s - 1e-9 and m["done_s"] >= m["admit_s"]
    steps = [m["step"] for m in meta]
    assert steps == sorted(steps)  # FIFO admission
    assert st.p99_ms >= st.p50_ms > 0


def test_served_vs_oracle(env):
    """A few requests of each kind against the oracle port's builtins."""
    import subprocess
    from horsepower_gb300.abi import Builtins, H_B, H_I, H_L
    from horsepower_gb300 import plans as P
    L, srv, (line, dim, fact, order) = env
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    ora = Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")
    h = lambda d: {k: L.to_py(v) for k, v in d.items()}
    hl, hd, hf, ho = h(line), h(dim), h(fact), h(order)
    reqs = [S.Request(S.FILTER_AGG, D.WIN_LO, D.WIN_HI, 0, 0, 0.0),
            S.Request(S.JOIN_GROUP, D.WIN_LO + 100, D.WIN_HI + 100, 0, 0, 0.0),
            S.Request(S.TOPK_ORDER, 0, 0, 5, 900, 0.0),
            S.Request(S.TOPK_ORDER, 0, 0, 20_000, 60_000, 0.0)]
    got, _, _ = srv.run(reqs)
    v = ora.to_py(P.filter_aggregate(ora, P.host_nodes(ora, hl, P.FILTER_TYPES)))[0]
    assert abs(got[0] - v) <= 1e-12 * abs(v)
    r = P.join_group(ora, P.host_nodes(ora, hd, P.DIM_TYPES), P.host_nodes(ora, hf, P.FACT_TYPES),
                     reqs[1].lo, reqs[1].hi)
    want = [ora.to_py(x) for x in r]
    g = got[1]
    assert np.array_equal(g[0], want[0].astype(np.int8)) and np.array_equal(g[5], want[5])
    for k in (2, 3, 4):
        assert np.allclose(g[k], want[k], rtol=1e-12, atol=0)
    for q, rows in zip(reqs[2:], got[2:]):
        key, sec = ho["key"], ho["sec"]
        m = ora.call("pfnAnd", ora.call("pfnGeq", ora.vec(key, H_L), ora.scalar(q.klo, H_L)),
                     ora.call("pfnLt", ora.vec(key, H_L), ora.scalar(q.khi, H_L)))
        w = ora.to_py(ora.call("pfnWhere", m))
        o = ora.to_py(ora.call("pfnOrderBy", ora.list([ora.vec(key[w], H_L), ora.vec(sec[w], H_I)]),
                               ora.vec(np.array([1, 1], bool), H_B)))
        assert np.array_equal(rows, w[o[:S.TOPK]]), q.klo
        ora.free_inputs()
