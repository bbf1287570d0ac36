"""Failure paths, made without faulting the GPU.

* A bounded device wait that runs out: hgpuSelfTestWait runs the library's
  own look-back wait functions over four tiles whose first tile never
  publishes (a flag nothing sets).  Every wait gives up after its poll
  limit, the call returns E_DEVICE_TIMEOUT (102) -- the code a builtin whose
  wait gave up returns -- and the library keeps working afterwards.
* Memory exhaustion: a child process caps the scratch arena
  (HGPU_SCRATCH_LIMIT_MB); a join that needs more scratch returns
  E_DEVICE_OOM (101) instead of exiting, and a small call after it works.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from horsepower_gb300.abi import H_E, H_I

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("mode", [0, 1])
def test_wait_times_out_and_library_recovers(mode):
    import horsepower_gb300
    L = horsepower_gb300.load()
    L.lib.hgpuSelfTestWait.restype = C.c_int32
    L.lib.hgpuSelfTestWait.argtypes = [C.c_int32, C.c_longlong]
    for _ in range(2):  # the error word is cleared by the read: a second run reports it again
        rc = L.lib.hgpuSelfTestWait(mode, 1 << 14)
        assert rc == 102, rc
        assert b"wait" in L.lib.hgpuLastError()
    x = np.arange(1, 100_001, dtype=np.float64)
    assert L.to_py(L.call("pfnSum", L.vec(x, H_E)))[0] == 5000050000.0
    assert L.lib.hgpuSelfTestWait(2, 10) == 1 and L.lib.hgpuSelfTestWait(0, 1 << 30) == 1  # E_DOMAIN
    L.free_inputs()


CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import horsepower_gb300
from horsepower_gb300.abi import H_I
L = horsepower_gb300.load()
rng = np.random.default_rng(1)
build = rng.permutation(40_000_000).astype(np.int32)[:8_000_000]
probe = rng.integers(0, 40_000_000, 30_000_000).astype(np.int32)
rc = L.rc("pfnJoinIndex", L.vec(build, H_I), L.vec(probe, H_I), L.sym("eq"))
print("join_rc", rc, L.lib.hgpuLastError().decode())
small = L.call("pfnJoinIndex", L.vec(np.array([3, 1, 2], np.int32), H_I), L.vec(np.array([1, 2, 3, 3], np.int32), H_I), L.sym("eq"))
print("small", sorted(zip(*[v.tolist() for v in L.to_py(small)])))
"""


def test_capped_scratch_arena_returns_oom():
    env = dict(os.environ, HGPU_SCRATCH_LIMIT_MB="64")
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    assert lines["join_rc"].startswith("101"), r.stdout
    # the linear join of a 3-row side: (row of [3, 1, 2], row of [1, 2, 3, 3]) pairs
    assert lines["small"] == "[(0, 2), (0, 3), (1, 0), (2, 1)]", r.stdout
