"""GB300-native HorseIR builtin library.

`load()` returns a `Builtins` handle on the in-tree libhgpu.so (the CUDA
library exporting the reference's pfn* C ABI).  There is no CPU fallback:
without the compiled library or a CUDA device, loading fails.
"""
import os

from .abi import Builtins, BuiltinError  # noqa: F401

PKG = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(PKG, "libhgpu.so")
_loaded = None


def load(build_if_missing=True):
    global _loaded
    if _loaded is not None:
        return _loaded
    if not os.path.exists(LIB):
        if not build_if_missing:
            raise RuntimeError("libhgpu.so is not built (python -m horsepower_gb300.build)")
        from .build import build
        build()
    lib = Builtins(LIB, "libhgpu")
    rc = lib.lib.hgpuSync()
    if rc:
        raise RuntimeError(f"libhgpu: CUDA unavailable ({lib.lib.hgpuLastError().decode()})")
    _loaded = lib
    return lib
