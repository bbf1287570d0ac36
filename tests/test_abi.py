"""The C-ABI library builds, loads without a GPU and exports every entry
point include/hgpu.h declares; without a device every builtin fails with
E_NO_DEVICE instead of falling back to the CPU."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hgpu.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(pfn\w+|hgpu\w+|initBackend|allocNode|initV|getHeapOffset|setHeapOffset|getTypeSize|getSymbol|getSymbolStr)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from horsepower_gb300.build import build
    path = build()
    return C.CDLL(path)


def test_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "horsepower_gb300", "libhgpu.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [n for n in declared() if n not in exported]
    assert not missing, f"declared in hgpu.h but not exported: {missing}"
    assert len(declared()) > 50


def test_compiled_queries_link_against_the_library(lib):
    """libhgpu_queries.so (queries/*.c) is built beside libhgpu.so, exports
    the compiled query and resolves the builtins it calls from libhgpu."""
    path = os.path.join(ROOT, "horsepower_gb300", "libhgpu_queries.so")
    assert os.path.exists(path)
    out = subprocess.run(["nm", "-D", path], capture_output=True, text=True, check=True).stdout
    assert any(ln.split()[-1] == "hgpuQueryJoinGroup" and " T " in ln for ln in out.splitlines())
    undefined = {ln.split()[-1] for ln in out.splitlines() if " U " in ln}
    assert {"pfnJoinIndex", "hgpuIndexMany", "hgpuGroupAggMany"} <= undefined
    assert C.CDLL(path).hgpuQueryJoinGroup


def test_sm103a_only(lib):
    # the build compiles for sm_103a only (one -gencode)
    from horsepower_gb300 import build as b
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_no_cpu_fallback_without_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from horsepower_gb300.abi import Builtins, H_B, H_E
    L = Builtins(os.path.join(ROOT, "horsepower_gb300", "libhgpu.so"), "libhgpu")
    rc = L.rc("pfnCompress", L.vec(np.array([True, False, True]), H_B), L.vec(np.array([1.0, 2.0, 3.0]), H_E))
    assert rc == 103  # E_NO_DEVICE
    with pytest.raises(RuntimeError):
        import horsepower_gb300
        horsepower_gb300._loaded = None
        horsepower_gb300.load()


def test_value_node_layout():
    from horsepower_gb300.abi import V0
    assert C.sizeof(V0) == 32
    assert V0.len.offset == 0 and V0.g.offset == 8 and V0.typ.offset == 16 and V0.u.offset == 24


def test_tuning_knob_ids_match_the_header():
    """The autotuner's knob ids are the HGPU_TUNE_* values include/hgpu.h
    defines, one for one."""
    from horsepower_gb300 import autotune as T
    src = open(HEADER).read()
    ids = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"#define\s+HGPU_TUNE_(\w+)\s+(\d+)", src)}
    assert ids and {k: v for k, (v, _) in T.KNOBS.items()} == ids
