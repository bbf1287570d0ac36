"""Build libhgpu.so (CUDA, sm_103a) in-tree.

    python -m horsepower_gb300.build          # or horsepower_gb300.build.build()

Every csrc/*.cu file is compiled in parallel with nvcc for sm_103a only and
linked into horsepower_gb300/libhgpu.so.  Objects go to horsepower_gb300/_build
and are rebuilt when a source or header changes.
"""
import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-Xptxas", "-O3",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "--expt-relaxed-constexpr"]


def _headers_digest():
    h = hashlib.sha1()
    for p in sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))):
        h.update(open(p, "rb").read())
    return h.hexdigest()


def _compile(src, hdr):
    base = os.path.splitext(os.path.basename(src))[0]
    obj = os.path.join(OUT, base + ".o")
    stamp = obj + ".sha"
    h = hashlib.sha1(open(src, "rb").read() + hdr.encode() + " ".join(_flags()).encode()).hexdigest()
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == h:
        return obj, False
    cmd = [nvcc()] + _flags() + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    open(stamp, "w").write(h)
    return obj, True


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr = _headers_digest()
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, hdr), srcs))
    objs = [o for o, _ in results]
    rebuilt = any(r for _, r in results)
    if rebuilt or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print(f"libhgpu.so: {len(srcs)} translation units ({'rebuilt' if rebuilt else 'up to date'})")
    build_queries(verbose)
    return LIB


QSRC = os.path.join(PKG, "queries")
QLIB = os.path.join(PKG, "libhgpu_queries.so")


def build_queries(verbose=False):
    """Compiled benchmark queries (callers of libhgpu, like the reference's
    generated query code) -> libhgpu_queries.so, linked against libhgpu.so."""
    srcs = sorted(glob.glob(os.path.join(QSRC, "*.c")))
    h = hashlib.sha1(b"".join(open(p, "rb").read() for p in srcs) + _headers_digest().encode()).hexdigest()
    stamp = os.path.join(OUT, "queries.sha")
    if os.path.exists(QLIB) and os.path.exists(stamp) and open(stamp).read() == h:
        return QLIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"), "-o", QLIB + ".tmp"] + srcs + \
          ["-L" + PKG, "-lhgpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"query build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(QLIB + ".tmp", QLIB)
    open(stamp, "w").write(h)
    if verbose:
        print(f"libhgpu_queries.so: {len(srcs)} queries")
    return QLIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
