"""Generate the ingest fixtures: CSV files, binary files written by the
reference's serializeV, and the values the reference's readCSV /
readSerializeV produce for them (tests/golden/ingest.npz).

Run where the HorsePower sources exist:
    make -C oracle ref
    python tests/golden/make_ingest.py
"""
import ctypes as C
import decimal
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from horsepower_gb300 import data as D  # noqa: E402
from horsepower_gb300.abi import Builtins, V0, table_columns  # noqa: E402
import ingest_cases as IC  # noqa: E402

OUT = os.path.join(HERE, "ingest")


def midpoint_texts():
    """Exact decimal expansions of rounding midpoints (ties go to even), the
    same texts with one more nonzero digit (just above) and with the last
    digit lowered (just below), for strtod (binary64) and strtof (binary32)."""
    decimal.getcontext().prec = 2000
    two = decimal.Decimal(2)
    mids = [two ** -1075,                            # 0 | smallest binary64 subnormal
            1 + two ** -53,                          # 1 | next binary64 after 1
            two ** 53 + 1,                           # integers above 2^53
            (2 - two ** -52) * two ** 1023 + two ** 970,  # largest binary64 | overflow
            1 + two ** -24,                          # binary32 after 1
            two ** -150,                             # 0 | smallest binary32 subnormal
            (2 - two ** -23) * two ** 127 + two ** 103]   # largest binary32 | overflow
    out = []
    for m in mids:
        mant, ex = format(m, "E").split("E")
        if "." not in mant:
            mant += ".0"
        out.append(f"{mant}e{ex}")
        out.append(f"{mant}1e{ex}")
        if mant[-1] != "0":
            out.append(f"{mant[:-1]}{int(mant[-1]) - 1}e{ex}")
    mant, ex = format(mids[1], "E").split("E")
    out.append(f"{mant}{'0' * 900}1e{ex}")  # a nonzero digit far past 800 significant digits
    out.append("1." + "0" * 900 + "1")
    return out


def main():
    os.makedirs(OUT, exist_ok=True)
    ref = Builtins(os.path.join(ROOT, "oracle", "_ref", "libref.so"), "reference")
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    ref.lib.readCSV.restype = C.c_void_p
    ref.lib.readCSV.argtypes = [C.c_char_p, C.c_longlong, C.c_void_p, C.c_void_p]
    ref.lib.serializeV.argtypes = [C.c_void_p, C.c_void_p]
    sep = C.c_char.in_dll(ref.lib, "LINE_SEP")
    hdr = C.c_bool.in_dll(ref.lib, "LINE_HEADER")
    maxline = C.c_longlong.in_dll(ref.lib, "LINE_MAX_CHAR")
    store = {}
    # CSV fixtures
    text, _ = D.lineitem_csv(1000, seed=3)
    files = {"lineitem_1k.tbl": text}
    files.update(IC.edge_files(midpoint_texts()))
    for name, body in files.items():
        open(os.path.join(OUT, name), "wb").write(body)
    tables = {}
    for case in IC.CSV_CASES:
        sep.value = case["sep"].encode()
        hdr.value = case["header"]
        maxline.value = case.get("maxline", 1024)
        types = (C.c_longlong * len(case["types"]))(*case["types"])
        syms = (C.c_longlong * len(case["types"]))(*[ref.lib.getSymbol(n.encode()) for n in case["names"]])
        t = ref.lib.readCSV(os.path.join(OUT, case["file"]).encode(), len(case["types"]), types, syms)
        node = V0.from_address(t)
        names, cols = table_columns(ref, node)
        IC.store_table(store, case["id"], names, cols)
        tables[case["id"]] = t
    sep.value = b"|"
    hdr.value = False
    maxline.value = 1024
    # binary fixtures written by the reference
    fp = libc.fopen(os.path.join(OUT, "lineitem_1k.bin").encode(), b"wb")
    ref.lib.serializeV(C.c_void_p(tables["lineitem"]), fp)
    libc.fclose(fp)
    vec_list, vec_expect = IC.vector_list(ref)
    fp = libc.fopen(os.path.join(OUT, "vectors.bin").encode(), b"wb")
    ref.lib.serializeV(C.addressof(vec_list), fp)
    libc.fclose(fp)
    IC.store_vectors(store, "vectors", vec_expect)
    np.savez_compressed(os.path.join(HERE, "ingest.npz"), **store)
    print("wrote", sorted(files), "and", len(store), "arrays")


if __name__ == "__main__":
    main()
