"""The documented mixed link: generated code or the interpreter linked first
against libhgpu, then against the reference's builtin library, which supplies
every builtin libhgpu does not export (h_primitive.h:72-211 declares 119,
libhgpu exports the accelerated ones).

A small C program is linked `-lhgpu -lref` (the reference library built here
from its sources as a shared library, as the integration guide prescribes)
and reports, through dladdr, which library each name bound to:
  * accelerated builtins (pfnCompress, pfnJoinIndex) -> libhgpu;
  * builtins only the reference has (pfnUnique, pfnVector) -> the reference;
  * the value entry points both define (initV, getHeapOffset) -> libhgpu,
    without a link conflict;
and that libhgpu then defaults to host residency, because the reference's
builtins read payloads on the host.  The same program linked against
libhgpu alone keeps outputs in HBM by default.  No GPU is used: the program
only resolves names and reads the residency.
"""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HGPU = os.path.join(ROOT, "horsepower_gb300")
REF = os.path.join(ROOT, "oracle", "_ref")

DRIVER = r"""
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdio.h>
#include <string.h>
#include "hgpu.h"
#ifdef WITH_REF
I pfnUnique(V z, V x);
I pfnVector(V z, V x, V y);
#endif
static const char *lib_of(void *f) {
    Dl_info i;
    if (!dladdr(f, &i) || !i.dli_fname) return "?";
    const char *s = strrchr(i.dli_fname, '/');
    return s ? s + 1 : i.dli_fname;
}
int main(void) {
    printf("pfnCompress %s\n", lib_of((void *)pfnCompress));
    printf("pfnJoinIndex %s\n", lib_of((void *)pfnJoinIndex));
#ifdef WITH_REF
    printf("pfnUnique %s\n", lib_of((void *)pfnUnique));
    printf("pfnVector %s\n", lib_of((void *)pfnVector));
#endif
    printf("initV %s\n", lib_of((void *)initV));
    printf("getHeapOffset %s\n", lib_of((void *)getHeapOffset));
    printf("residency %d\n", hgpuGetResidency());
    return 0;
}
"""


def _build_and_run(tmp, with_ref):
    src = os.path.join(tmp, "driver.c")
    exe = os.path.join(tmp, "driver_ref" if with_ref else "driver_alone")
    with open(src, "w") as f:
        f.write(DRIVER)
    cmd = ["gcc", "-O1", "-I" + os.path.join(ROOT, "include"), src, "-o", exe, "-L" + HGPU, "-lhgpu",
           "-Wl,-rpath," + HGPU, "-ldl"]
    if with_ref:
        cmd[2:2] = ["-DWITH_REF"]
        cmd += ["-L" + REF, "-lref", "-Wl,-rpath," + REF]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    env = {k: v for k, v in os.environ.items() if k != "HGPU_RESIDENCY"}
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60, env=env)
    assert r.returncode == 0, r.stderr
    return dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())


@pytest.mark.skipif(not os.path.exists(os.path.join(HGPU, "libhgpu.so")), reason="libhgpu not built")
@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "libref.so")), reason="the reference library is built only where its sources are")
def test_mixed_link_binds_each_builtin_to_its_library():
    with tempfile.TemporaryDirectory() as tmp:
        got = _build_and_run(tmp, True)
    assert got["pfnCompress"] == "libhgpu.so" and got["pfnJoinIndex"] == "libhgpu.so"
    assert got["pfnUnique"] == "libref.so" and got["pfnVector"] == "libref.so"
    assert got["initV"] == "libhgpu.so" and got["getHeapOffset"] == "libhgpu.so"
    assert got["residency"] == "1"  # HGPU_RESIDENT_HOST: the reference's builtins read payloads on the host


@pytest.mark.skipif(not os.path.exists(os.path.join(HGPU, "libhgpu.so")), reason="libhgpu not built")
def test_alone_outputs_stay_in_hbm():
    with tempfile.TemporaryDirectory() as tmp:
        got = _build_and_run(tmp, False)
    assert got["pfnCompress"] == "libhgpu.so"
    assert got["residency"] == "0"  # HGPU_RESIDENT_DEVICE
