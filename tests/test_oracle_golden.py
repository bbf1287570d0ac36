"""The CPU oracle port reproduces the reference library's golden vectors.

golden.npz holds inputs and outputs produced by the reference's own builtin
library (compiled from its sources by oracle/Makefile `ref`); this pins the
oracle that the GPU parity tests use.
"""
import os
import subprocess

import pytest

import runner
from horsepower_gb300.abi import Builtins

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


@pytest.fixture(scope="module")
def oracle():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")


CASES = runner.load(GOLDEN)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference(oracle, case):
    if case["rc"]:
        rc = oracle.rc(case["fn"], *[runner.build_arg(oracle, a) for a in case["args"]])
        assert rc == case["rc"]
        return
    rc, obj = runner.run_case(oracle, case)
    exact = dict(case, canonical=False)  # the oracle restates the quicksort: always exact
    runner.compare(exact, rc, obj)
    oracle.free_inputs()


def test_oracle_fused_group_aggregates_match_chain(oracle):
    for case in CASES:
        if case["fn"] != "@chain_group_agg":
            continue
        rc, obj = runner.run_case(oracle, case, fused=True)
        runner.compare(case, rc, obj)


def test_oracle_index_many_is_separate_index(oracle):
    """The oracle's hgpuIndexMany (the common index pattern, pattern.cc:558-672)
    is one pfnIndex per column: the checker the GPU path is compared with."""
    import ctypes as C
    import numpy as np
    from horsepower_gb300.abi import H_E, H_I, H_L
    rng = np.random.default_rng(3)
    cols = [(H_E, rng.standard_normal(500)), (H_I, rng.integers(-9, 9, 500).astype(np.int32))]
    idx = oracle.vec(rng.integers(0, 500, 1000), H_L)
    xs = [oracle.vec(a, t) for t, a in cols]
    zs = [oracle.node() for _ in xs]
    fn = oracle.lib.hgpuIndexMany
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong]
    assert fn(oracle.node_array(zs), oracle.node_array(xs), C.byref(idx), 2) == 0
    for z, x in zip(zs, xs):
        want = oracle.to_py(oracle.call("pfnIndex", x, idx))
        assert oracle.to_py(z).tobytes() == want.tobytes()
    oracle.free_inputs()


def test_compiled_query_source_is_warning_free():
    """queries/join_group.c compiles cleanly against include/hgpu.h."""
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = os.path.join(root, "horsepower_gb300", "queries", "join_group.c")
    r = subprocess.run(["gcc", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(root, "include"), src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
