"""Symbols and strings on the GPU: @like and symbol compares against the
oracle (whose results are pinned to the reference's own PCRE2 @like and
compareSymbol by the golden fixtures), on a 1M-row lineitem table read by
the GPU CSV reader, whose string column is matched in HBM."""
import os

import numpy as np
import pytest

from ingest_run import Ingest
from horsepower_gb300 import data as D
from horsepower_gb300.abi import Builtins, V0, table_columns

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tables(tmp_path_factory):
    import subprocess
    import horsepower_gb300
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    gpu = horsepower_gb300.load()
    ora = Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")
    text, _ = D.lineitem_csv(1_000_000, seed=21)
    p = tmp_path_factory.mktemp("strings") / "lineitem.tbl"
    p.write_bytes(text)
    out = []
    for lib in (gpu, ora):
        rc, t = Ingest(lib).csv(str(p), D.LINEITEM_TYPES, D.LINEITEM_NAMES)
        assert rc == 0
        out.append((lib, t))
    return out


def column(t, j):
    vals = V0.from_address(t.g + 32)
    return V0.from_address(vals.g + 32 * j)


@pytest.mark.parametrize("pat", [b"%special%", b"%a%b%c%", b"x%", b"%zz", b"___ %", b"%", b"a%e%i%o%u%"])
def test_like_on_loaded_strings(tables, pat):
    outs = []
    for lib, t in tables:
        z = lib.call("pfnLike", column(t, 15), lib.strs([pat]))
        outs.append(lib.to_py(z))
    assert outs[0].dtype == np.bool_ and np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("pat", ["%AIR%", "R%", "%L", "_A%", "SHIP"])
def test_like_on_symbols(tables, pat):
    outs = [lib.to_py(lib.call("pfnLike", column(t, 14), lib.sym(pat))) for lib, t in tables]
    assert np.array_equal(outs[0], outs[1])
    names = table_columns(tables[0][0], tables[0][1])[1][14]
    import fnmatch
    want = np.array([fnmatch.fnmatchcase(s, pat.replace("%", "*").replace("_", "?")) for s in names])
    assert np.array_equal(outs[0], want)


@pytest.mark.parametrize("op", ["pfnLt", "pfnLeq", "pfnGt", "pfnGeq", "pfnEq", "pfnNeq"])
def test_symbol_compares(tables, op):
    outs = []
    for lib, t in tables:
        a = lib.to_py(lib.call(op, column(t, 14), lib.sym("MAIL")))
        b = lib.to_py(lib.call(op, column(t, 13), column(t, 14)))
        outs.append((a, b))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    names = table_columns(tables[0][0], tables[0][1])[1]
    cmp = {"pfnLt": lambda u, v: u < v, "pfnLeq": lambda u, v: u <= v, "pfnGt": lambda u, v: u > v,
           "pfnGeq": lambda u, v: u >= v, "pfnEq": lambda u, v: u == v, "pfnNeq": lambda u, v: u != v}[op]
    want = np.array([cmp(s.encode(), b"MAIL") for s in names[14]])
    assert np.array_equal(outs[0][0], want)


def test_like_errors_match_oracle(tables):
    for lib, t in tables:
        col = column(t, 15)
        assert lib.rc("pfnLike", col, lib.strs([b""])) == 7            # E_NULL_VALUE
        assert lib.rc("pfnLike", col, lib.strs([b"a(b)%"])) == 99      # a regex operator in the translated pattern
        assert lib.rc("pfnLike", lib.strs([b"a", b"b"]), lib.strs([b"a", b"%"])) == 99  # one pattern per row
        assert lib.rc("pfnLike", lib.strs([b"a", b"b", b"c"]), lib.strs([b"a", b"%"])) == 5
