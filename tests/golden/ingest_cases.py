"""Ingest fixtures shared by make_ingest.py (which runs them through the
reference's readCSV / serializeV) and the tests (which replay them through
the oracle and libhgpu).

CSV cases follow loadItem's conversions (h_io.cc:164-181): atoi / atol with
strtol's clamping, strtof / strtod (ties-to-even, subnormals, overflow,
inf/nan, texts past 800 significant digits), first character, %d-%d-%d
dates, symbols and strings; fields are trimmed as getField does.
"""
import ctypes as C

import numpy as np

from horsepower_gb300 import data as D
from horsepower_gb300.abi import H_B, H_C, H_D, H_E, H_F, H_G, H_H, H_I, H_J, H_L, H_Q, H_S, V0

FLOATS = ["0", "-0", "0.0", "1", "-1", "3.14159", "1e10", "1E-5", "+.5", "5.", "-.5e-3", "  7.25", "\t2.5", "1e",
          "1e+", "abc", "", ".", "-", "inf", "-INF", "Infinity", "nan", "-nan", "NaN", "0.1", "0.3", "2.675",
          "123456789012345678", "0.12345678901234567", "1.7976931348623157e308", "1.7976931348623158e308",
          "1.7976931348623159e308", "1e309", "-1e400", "1e-400", "4.9406564584124654e-324",
          "2.4703282292062327e-324", "2.4703282292062328e-324", "2.2250738585072011e-308",
          "2.2250738585072014e-308", "3.4028235e38", "3.4028236e38", "1.4e-45", "7e-46", "8e-46", "1.17549435e-38",
          "16777217", "16777219", "1234567890" * 6, "0." + "0" * 300 + "1234567", "9" * 400, "1" + "0" * 310,
          "0.000000000000000000000000000000000000000000001401298464324817"]
LONGS = ["0", "-0", "+7", "  42", "\t5", "12abc", "", "abc", "9223372036854775807", "9223372036854775808",
         "-9223372036854775808", "-9223372036854775809", "99999999999999999999999", "--5", "+-5", "0x10", "1e5"]
INTS = ["2147483647", "2147483648", "4294967297", "-2147483649", "99999999999999999999", "-7", " 3 "]
BYTES = ["127", "128", "255", "-129", "1000", "0"]
SHORTS = ["32767", "32768", "70000", "-40000"]
BOOLS = ["0", "1", "2", "-1", "abc", "256"]
CHARS = ["x", "", "  y", "zz", "7"]
DATES = ["1994-01-01", "1994-1-1", "  1994-01-01", "1994-01-01junk", "-5-3-2", "+1994-+1-+1", "1994- 01- 01",
         "2000-12-31"]

NUM_TYPES = [H_E, H_F, H_L, H_I, H_J, H_H, H_B, H_C, H_D]
CSV_CASES = [
    dict(id="lineitem", file="lineitem_1k.tbl", sep="|", header=False, types=D.LINEITEM_TYPES,
         names=D.LINEITEM_NAMES),
    dict(id="numbers", file="numbers.tbl", sep="|", header=False, types=NUM_TYPES, maxline=4096,
         names=["e", "f", "l", "i", "j", "h", "b", "c", "d"]),
    dict(id="spaces", file="spaces.txt", sep=" ", header=True, types=[H_E, H_E, H_C, H_I],
         names=["sptprice", "strike", "optiontype", "n"]),
    dict(id="crlf", file="crlf.tbl", sep="|", header=False, types=[H_I, H_Q, H_S], names=["k", "mode", "note"]),
]


def edge_files(extra_floats):
    """The edge-case CSV files (bytes), given the midpoint texts."""
    floats = FLOATS + list(extra_floats)
    cols = [floats, floats, LONGS, INTS, BYTES, SHORTS, BOOLS, CHARS, DATES]
    n = max(len(c) for c in cols)
    lines = ["|".join(c[i % len(c)] for c in cols) + "|" for i in range(n)]
    numbers = ("\n".join(lines) + "\n").encode()
    spaces = b"sptprice strike optiontype n\n" + b"".join(
        f"{42.5 + i / 8} {40 + i} {'CP'[i % 2]} {i * 3 - 5}\n".encode() for i in range(40))
    crlf = (b"1|AIR|hello world|\r\n2|RAIL|  spaced   out  |\r\n3|AIR||\r\n4|TRUCK|last line|\r\n"
            b"5|RAIL|no newline at the end|")
    return {"numbers.tbl": numbers, "spaces.txt": spaces, "crlf.tbl": crlf}


def _put_column(store, key, col):
    if isinstance(col, np.ndarray):
        store[key] = col
    elif col and isinstance(col[0], str):
        store[key + ".sym"] = np.array(col, dtype=str)
    else:
        store[key + ".str"] = np.frombuffer(b"".join(col), np.uint8) if col else np.zeros(0, np.uint8)
        store[key + ".len"] = np.array([len(c) for c in col], np.int64)


def _get_column(z, key):
    if key in z.files:
        return z[key]
    if key + ".sym" in z.files:
        return [str(s) for s in z[key + ".sym"]]
    raw, lens = z[key + ".str"].tobytes(), z[key + ".len"]
    out, o = [], 0
    for n in lens:
        out.append(raw[o:o + n])
        o += n
    return out


def store_table(store, tid, names, cols):
    store[f"{tid}/names"] = np.array(names, dtype=str)
    for j, c in enumerate(cols):
        _put_column(store, f"{tid}/c{j}", c)


def load_table(z, tid):
    names = [str(s) for s in z[f"{tid}/names"]]
    return names, [_get_column(z, f"{tid}/c{j}") for j in range(len(names))]


def same_column(a, b):
    if isinstance(b, np.ndarray):
        a = np.asarray(a)
        if a.dtype != b.dtype or a.shape != b.shape:
            return False
        if b.dtype.kind == "f":  # bit patterns: -0, NaN signs
            return np.array_equal(a.view(np.uint8), b.view(np.uint8))
        return np.array_equal(a, b)
    return list(a) == list(b)


def assert_same_table(got, want, what=""):
    (gn, gc), (wn, wc) = got, want
    assert gn == wn, f"{what}: names {gn} != {wn}"
    for j, (a, b) in enumerate(zip(gc, wc)):
        assert same_column(a, b), f"{what}: column {wn[j]} differs"


def vector_list(lib):
    """A list node of assorted vectors (inline, empty, char, symbol, string,
    date, list) built with `lib`, and its expected python form."""
    rng = np.random.default_rng(11)
    items, expect = [], []
    for typ, arr in [(H_I, rng.integers(-1000, 1000, 1000).astype(np.int32)), (H_E, np.array([2.5])),
                     (H_L, np.zeros(0, np.int64)), (H_B, np.array([True, False, True])),
                     (H_D, np.array([19940101, 19981231], np.int32)), (H_C, np.frombuffer(b"hello", np.int8)),
                     (H_E, rng.standard_normal(3000))]:
        items.append(lib.vec(arr, typ))
        expect.append(("vec", typ, arr))
    items.append(lib.syms(["a", "bb", "a", "ccc"]))
    expect.append(("sym", ["a", "bb", "a", "ccc"]))
    texts = [b"first", b"", b"third text"]
    bufs = [C.create_string_buffer(t) for t in texts]
    ptrs = (C.c_void_p * len(texts))(*[C.addressof(b) for b in bufs])
    s = V0()
    s.typ, s.len, s.g = H_S, len(texts), C.addressof(ptrs)
    lib._keep.append((s, bufs, ptrs))
    items.append(s)
    expect.append(("str", texts))
    inner = lib.list([lib.vec(np.arange(5, dtype=np.int64), H_L), lib.syms(["x"])])
    items.append(inner)
    expect.append(("list", [("vec", H_L, np.arange(5, dtype=np.int64)), ("sym", ["x"])]))
    return lib.list(items), expect


def node_to_py(lib, v):
    if v.typ == H_G:
        return ("list", [node_to_py(lib, V0.from_address(v.g + 32 * i)) for i in range(v.len)])
    if v.typ == H_Q:
        return ("sym", [lib.lib.getSymbolStr(int(i)).decode() for i in np.atleast_1d(lib.to_py(v))])
    if v.typ == H_S:
        ptrs = [v.i64] if v.len == 1 else list((C.c_uint64 * v.len).from_address(v.g)) if v.len else []
        return ("str", [C.string_at(p) for p in ptrs])
    return ("vec", v.typ, np.atleast_1d(lib.to_py(v)))


def assert_same_node(got, want, path="x"):
    assert got[0] == want[0], f"{path}: kind {got[0]} != {want[0]}"
    if got[0] == "list":
        assert len(got[1]) == len(want[1]), f"{path}: list length"
        for i, (a, b) in enumerate(zip(got[1], want[1])):
            assert_same_node(a, b, f"{path}[{i}]")
    elif got[0] == "vec":
        assert got[1] == want[1], f"{path}: type {got[1]} != {want[1]}"
        assert same_column(np.asarray(got[2]).astype(np.asarray(want[2]).dtype), np.asarray(want[2])), f"{path}: values"
    else:
        assert list(got[1]) == list(want[1]), f"{path}: {got[1]} != {want[1]}"


def store_vectors(store, vid, expect):
    def rec(prefix, e):
        if e[0] == "list":
            store[prefix + ".list"] = np.array(len(e[1]))
            for i, x in enumerate(e[1]):
                rec(f"{prefix}.{i}", x)
        elif e[0] == "vec":
            store[prefix + ".vec"] = np.asarray(e[2])
            store[prefix + ".typ"] = np.array(e[1])
        elif e[0] == "sym":
            store[prefix + ".sym"] = np.array(e[1], dtype=str)
        else:
            _put_column(store, prefix, list(e[1]))
    rec(vid, ("list", expect))


def load_vectors(z, vid):
    def rec(prefix):
        if prefix + ".list" in z.files:
            return ("list", [rec(f"{prefix}.{i}") for i in range(int(z[prefix + ".list"]))])
        if prefix + ".vec" in z.files:
            return ("vec", int(z[prefix + ".typ"]), z[prefix + ".vec"])
        if prefix + ".sym" in z.files:
            return ("sym", [str(s) for s in z[prefix + ".sym"]])
        return ("str", _get_column(z, prefix))
    return rec(vid)
