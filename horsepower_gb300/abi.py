"""ctypes binding of the HorseIR builtin C ABI (include/hgpu.h).

One `Builtins` object wraps one shared library that exports the reference's
`I pfnXxx(V z, V x, ...)` entry points over the `V0` value node
(src/horseir/v3/backend/common.h:31-55).  The same class drives the GPU
library (libhgpu.so), so a sequence of builtin calls written once runs
unchanged against any library with this ABI.

Host vectors are built from numpy arrays (the array must stay alive while
the node is used; `Builtins` keeps a reference).  Results are read back with
`to_py`, which copies device-resident payloads to the host through
`hgpuToHost` when the library provides it.
"""
import ctypes as C
import os

import numpy as np

H_B, H_J, H_H, H_I, H_L, H_F, H_E, H_X, H_C, H_Q, H_S = 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10
H_M, H_D, H_Z, H_U, H_W, H_T, H_G, H_N, H_Y = 11, 12, 13, 14, 15, 16, 17, 18, 19
H_A = 90

DTYPE = {
    H_B: np.bool_, H_J: np.int8, H_H: np.int16, H_I: np.int32, H_L: np.int64,
    H_F: np.float32, H_E: np.float64, H_C: np.int8, H_Q: np.int64,
    H_M: np.int32, H_D: np.int32, H_Z: np.int64, H_U: np.int32, H_W: np.int32, H_T: np.int32,
}
TYPE_OF = {np.dtype(np.bool_): H_B, np.dtype(np.int8): H_J, np.dtype(np.int16): H_H,
           np.dtype(np.int32): H_I, np.dtype(np.int64): H_L, np.dtype(np.float32): H_F,
           np.dtype(np.float64): H_E}
ERR = {1: "E_DOMAIN", 2: "E_GENERAL", 3: "E_INDEX", 4: "E_DIV_ZERO", 5: "E_LENGTH", 6: "E_TYPE",
       9: "E_MATCH", 10: "E_ENUM_INDEX", 11: "E_RAZE_LIST", 12: "E_UNKNOWN", 99: "E_NOT_IMPL", 100: "E_DEVICE",
       101: "E_DEVICE_OOM", 102: "E_DEVICE_TIMEOUT", 103: "E_NO_DEVICE", 104: "E_ADMISSION",
       105: "E_CANCELLED"}


class _U(C.Union):
    _fields_ = [("b", C.c_bool), ("j", C.c_int8), ("h", C.c_int16), ("i32", C.c_int32),
                ("i64", C.c_longlong), ("f32", C.c_float), ("f64", C.c_double), ("p", C.c_void_p)]


class V0(C.Structure):
    _anonymous_ = ("u",)
    _fields_ = [("len", C.c_longlong), ("g", C.c_void_p), ("typ", C.c_int32), ("u", _U)]


assert C.sizeof(V0) == 32
PV = C.POINTER(V0)


class BuiltinError(RuntimeError):
    def __init__(self, name, code, detail=""):
        super().__init__(f"{name} returned {code} ({ERR.get(code, '?')}) {detail}".strip())
        self.code = code


_MONADIC = ["pfnWhere", "pfnSum", "pfnAvg", "pfnMin", "pfnMax", "pfnLen", "pfnNot", "pfnGroup",
            "pfnGroupTrie", "pfnGroupBasic", "pfnKeys", "pfnValues", "pfnRaze"]
_DYADIC = ["pfnCompress", "pfnLt", "pfnLeq", "pfnGt", "pfnGeq", "pfnEq", "pfnNeq", "pfnPlus",
           "pfnMinus", "pfnMul", "pfnDiv", "pfnAnd", "pfnNand", "pfnOr", "pfnNor", "pfnXor",
           "pfnIndex", "pfnIndexOf", "pfnMember", "pfnOrderBy", "hgpuGroupSum", "hgpuGroupAvg",
           "hgpuGroupMin", "hgpuGroupMax", "hgpuGroupLen"]
FUNC1 = C.CFUNCTYPE(C.c_int32, PV, PV)
FUNC2 = C.CFUNCTYPE(C.c_int32, PV, PV, PV)


class Builtins:
    """A builtin library reached through the pfn* C ABI."""

    def __init__(self, path, name=None):
        self.path = os.path.abspath(path)
        self.name = name or os.path.basename(path)
        self.lib = C.CDLL(self.path, mode=os.RTLD_LOCAL | os.RTLD_NOW)
        L = self.lib
        for f in _MONADIC:
            if hasattr(L, f):
                getattr(L, f).restype = C.c_int32
                getattr(L, f).argtypes = [PV, PV]
        for f in _DYADIC:
            if hasattr(L, f):
                getattr(L, f).restype = C.c_int32
                getattr(L, f).argtypes = [PV, PV, PV]
        for f, at in [("pfnJoinIndex", [PV, PV, PV, PV]), ("pfnCompare", [PV, PV, PV, C.c_int32]),
                      ("pfnArith", [PV, PV, PV, C.c_int32]), ("pfnReduce", [PV, PV, C.c_int32]),
                      ("pfnList", [PV, C.c_longlong, C.POINTER(PV)]), ("pfnEach", [PV, PV, C.c_void_p]),
                      ("pfnEachRight", [PV, PV, PV, C.c_void_p])]:
            if hasattr(L, f):
                getattr(L, f).restype = C.c_int32
                getattr(L, f).argtypes = at
        L.getSymbol.restype = C.c_longlong
        L.getSymbol.argtypes = [C.c_char_p]
        L.getHeapOffset.restype = C.c_longlong
        L.setHeapOffset.restype = C.c_longlong
        L.setHeapOffset.argtypes = [C.c_longlong]
        self.has_device = hasattr(L, "hgpuToHost")
        if self.has_device:
            L.hgpuToHost.restype = C.c_int32
            L.hgpuToHost.argtypes = [PV, PV]
            L.hgpuIsDevice.restype = C.c_int32
            L.hgpuIsDevice.argtypes = [PV]
            L.hgpuLastError.restype = C.c_char_p
        L.getSymbolStr.restype = C.c_char_p
        L.getSymbolStr.argtypes = [C.c_longlong]
        L.initBackend()
        self._keep = []

    # ------------------------------------------------------------ values
    def node(self):
        v = V0()
        self._keep.append(v)
        return v

    def node_array(self, nodes):
        """A `V *` array over nodes (kept alive by this object)."""
        arr = (PV * max(len(nodes), 1))(*[C.pointer(v) for v in nodes])
        self._keep.append(arr)
        return arr

    def vec(self, arr, typ=None):
        """A host vector node over a numpy array (kept alive by this object)."""
        arr = np.ascontiguousarray(arr)
        if typ is None:
            typ = TYPE_OF[arr.dtype]
        want = np.dtype(DTYPE[typ])
        if arr.dtype != want:
            arr = arr.astype(want)
        v = V0()
        v.typ, v.len = typ, arr.size
        if arr.size <= 1:
            C.memmove(C.addressof(v) + V0.u.offset, arr.ctypes.data, arr.nbytes)
            v.g = C.addressof(v) + V0.u.offset
        else:
            v.g = arr.ctypes.data
        self._keep.append((v, arr))
        return v

    def scalar(self, value, typ):
        return self.vec(np.array([value], dtype=DTYPE[typ]), typ)

    def sym(self, name):
        v = V0()
        v.typ, v.len = H_Q, 1
        v.i64 = self.lib.getSymbol(name.encode())
        v.g = C.addressof(v) + V0.u.offset
        self._keep.append(v)
        return v

    def syms(self, names):
        """A symbol vector (H_Q) of several names, e.g. the ops of a multi-column join."""
        ids = np.array([self.lib.getSymbol(n.encode()) for n in names], dtype=np.int64)
        return self.vec(ids, H_Q)

    def strs(self, texts):
        """A string vector (H_S): host pointers to NUL-terminated copies of `texts` (bytes)."""
        bufs = [C.create_string_buffer(t) for t in texts]
        ptrs = (C.c_void_p * max(len(texts), 1))(*[C.addressof(b) for b in bufs])
        v = V0()
        v.typ, v.len = H_S, len(texts)
        if len(texts) <= 1:
            if texts:
                v.i64 = C.addressof(bufs[0])
            v.g = C.addressof(v) + V0.u.offset
        else:
            v.g = C.addressof(ptrs)
        self._keep.append((v, bufs, ptrs))
        return v

    def chars(self, text):
        """A char vector (H_C) over `text` (bytes), NUL after the last character."""
        arr = np.frombuffer(text + b"\0", np.int8)
        v = V0()
        v.typ, v.len = H_C, len(text)
        if len(text) <= 1:
            C.memmove(C.addressof(v) + V0.u.offset, arr.ctypes.data, arr.nbytes)
            v.g = C.addressof(v) + V0.u.offset
        else:
            v.g = arr.ctypes.data
        self._keep.append((v, arr))
        return v

    def list(self, items, typ=H_G):
        arr = (V0 * max(len(items), 1))()
        for i, it in enumerate(items):
            C.memmove(C.addressof(arr) + i * 32, C.addressof(it), 32)
            if it.len <= 1 and it.typ in DTYPE and it.g == C.addressof(it) + V0.u.offset:
                arr[i].g = C.addressof(arr) + i * 32 + V0.u.offset
        v = V0()
        v.typ, v.len, v.g = typ, len(items), C.addressof(arr)
        self._keep.append((v, arr, items))
        return v

    def free_inputs(self):
        self._keep = []

    # ------------------------------------------------------------- calls
    def call(self, fname, *args, check=True):
        z = self.node()
        fn = getattr(self.lib, fname)
        conv = [C.byref(a) if isinstance(a, V0) else a for a in args]
        rc = fn(C.byref(z), *conv)
        if rc and check:
            detail = ""
            if self.has_device:
                msg = self.lib.hgpuLastError()
                detail = msg.decode() if msg else ""
            raise BuiltinError(fname, rc, detail)
        return z if not rc else rc

    def rc(self, fname, *args):
        """Call and return only the status code."""
        z = self.node()
        fn = getattr(self.lib, fname)
        conv = [C.byref(a) if isinstance(a, V0) else a for a in args]
        return fn(C.byref(z), *conv)

    def fn_ptr(self, fname):
        return C.cast(getattr(self.lib, fname), C.c_void_p).value

    # -------------------------------------------------------------- read
    def to_py(self, v):
        """Copy a node (recursively) into numpy arrays / python lists."""
        if v.typ in (H_G, H_N):
            out = [self.to_py(V0.from_address(v.g + 32 * i)) for i in range(v.len)]
            return ("dict", out[0], out[1]) if v.typ == H_N else out
        if self.has_device and v.typ in DTYPE and v.len > 1 and self.lib.hgpuIsDevice(C.byref(v)):
            h = V0()
            rc = self.lib.hgpuToHost(C.byref(h), C.byref(v))
            if rc:
                raise BuiltinError("hgpuToHost", rc, (self.lib.hgpuLastError() or b"").decode())
            return _read_host(h)
        return _read_host(v)


def table_columns(lib, t):
    """An H_A table node -> (column names, columns).  Numeric columns come back
    as numpy arrays, symbols as lists of str, strings as lists of bytes."""
    assert t.typ == H_A, t.typ
    keys = V0.from_address(t.g)
    vals = V0.from_address(t.g + 32)
    names = [lib.lib.getSymbolStr(int(i)).decode() for i in np.atleast_1d(lib.to_py(keys))]
    cols = []
    for j in range(vals.len):
        c = V0.from_address(vals.g + 32 * j)
        if c.typ == H_Q:
            cols.append([lib.lib.getSymbolStr(int(i)).decode() for i in lib.to_py(c)])
        elif c.typ == H_S:
            ptrs = [c.i64] if c.len == 1 else list((C.c_uint64 * c.len).from_address(c.g)) if c.len else []
            cols.append([C.string_at(p) for p in ptrs])
        else:
            cols.append(lib.to_py(c))
    return names, cols


def _read_host(v):
    typ, n = v.typ, v.len
    if typ in DTYPE:
        dt = np.dtype(DTYPE[typ])
        if n == 0:
            return np.zeros(0, dt)
        buf = (C.c_char * (n * dt.itemsize)).from_address(v.g)
        return np.frombuffer(buf, dt).copy()
    if typ in (H_G, H_N):
        out = []
        for i in range(n):
            e = V0.from_address(v.g + 32 * i)
            out.append(_read_host(e))
        return ("dict", out[0], out[1]) if typ == H_N else out
    raise ValueError(f"cannot read type {typ}")
