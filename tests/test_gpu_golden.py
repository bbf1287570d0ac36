"""libhgpu reproduces the reference library's golden vectors (GPU parity).

Inputs and expected outputs come from golden.npz, produced by the reference's
own builtin library.  Integer, index, boolean and permutation outputs must be
bit-exact; f64 aggregates match within the case's relative tolerance
(1e-12); cases built on the reference's unstable quicksort are compared as
partitions / ordered values (`canonical`).
"""
import os

import pytest

import runner

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = runner.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))


@pytest.fixture(scope="module")
def gpu():
    import horsepower_gb300
    return horsepower_gb300.load()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_gpu_matches_reference(gpu, case):
    if case["rc"]:
        rc = gpu.rc(case["fn"], *[runner.build_arg(gpu, a) for a in case["args"]])
        assert rc == case["rc"]
        return
    rc, obj = runner.run_case(gpu, case)
    runner.compare(case, rc, obj)
    gpu.free_inputs()


def test_gpu_fused_group_aggregates(gpu):
    for case in CASES:
        if case["fn"] != "@chain_group_agg":
            continue
        rc, obj = runner.run_case(gpu, case, fused=True)
        runner.compare(case, rc, obj)
