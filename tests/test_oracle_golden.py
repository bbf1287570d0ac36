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
