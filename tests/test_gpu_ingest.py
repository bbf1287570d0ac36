"""GPU table ingest against the reference's own loader results and the
oracle: readCSV parsed on the GPU (every fixture bit-exact, including the
float edge cases), binary tables written by the reference read into HBM,
binary files written here read back by the oracle, the reference's
undefined cases as errors, and a 1M-row lineitem-shaped file checked
against the values its generator knows exactly."""
import ctypes as C
import os

import numpy as np
import pytest

import ingest_cases as IC
from ingest_run import FIXTURES, Ingest
from horsepower_gb300 import data as D
from horsepower_gb300.abi import Builtins, H_E, H_F, table_columns

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXPECT = np.load(os.path.join(ROOT, "tests", "golden", "ingest.npz"))


@pytest.fixture(scope="module")
def libs():
    import subprocess
    import horsepower_gb300
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    gpu = horsepower_gb300.load()
    ora = Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")
    return (gpu, Ingest(gpu)), (ora, Ingest(ora))


@pytest.mark.parametrize("case", IC.CSV_CASES, ids=[c["id"] for c in IC.CSV_CASES])
def test_csv_matches_reference(libs, case):
    (gpu, ing), _ = libs
    rc, t = ing.case(case)
    assert rc == 0, gpu.lib.hgpuLastError()
    IC.assert_same_table(table_columns(gpu, t), IC.load_table(EXPECT, case["id"]), case["id"])


def test_reads_reference_binaries(libs):
    (gpu, ing), _ = libs
    rc, t = ing.load(os.path.join(FIXTURES, "lineitem_1k.bin"))
    assert rc == 0, gpu.lib.hgpuLastError()
    IC.assert_same_table(table_columns(gpu, t), IC.load_table(EXPECT, "lineitem"), "lineitem.bin")
    rc, v = ing.load(os.path.join(FIXTURES, "vectors.bin"))
    assert rc == 0, gpu.lib.hgpuLastError()
    IC.assert_same_node(IC.node_to_py(gpu, v), IC.load_vectors(EXPECT, "vectors"))


def test_binaries_cross_read_with_oracle(libs, tmp_path):
    (gpu, ing), (ora, oing) = libs
    rc, t = ing.load(os.path.join(FIXTURES, "lineitem_1k.bin"))
    assert rc == 0
    p = str(tmp_path / "gpu.bin")
    assert ing.save(p, t) == 0, gpu.lib.hgpuLastError()
    rc, t2 = oing.load(p)
    assert rc == 0
    IC.assert_same_table(table_columns(ora, t2), IC.load_table(EXPECT, "lineitem"), "written here, read by the oracle")
    rc, v = oing.load(os.path.join(FIXTURES, "vectors.bin"))
    assert rc == 0
    q = str(tmp_path / "ora.bin")
    assert oing.save(q, v) == 0
    rc, v2 = ing.load(q)
    assert rc == 0, gpu.lib.hgpuLastError()
    IC.assert_same_node(IC.node_to_py(gpu, v2), IC.load_vectors(EXPECT, "vectors"))
    r = str(tmp_path / "gpu_vec.bin")
    assert ing.save(r, v2) == 0
    rc, v3 = oing.load(r)
    assert rc == 0
    IC.assert_same_node(IC.node_to_py(ora, v3), IC.load_vectors(EXPECT, "vectors"))


def test_csv_errors_match_oracle(libs, tmp_path):
    bad = {"fields.tbl": (b"1|2|\n3|\n", [3, 3]), "long.tbl": (b"1|" + b"7" * 1100 + b"|\n", [3, 3]),
           "nul.tbl": (b"1|2\x003|\n", [3, 3]), "date.tbl": (b"1994/01/01|\n", [12]),
           "hex.tbl": (b"0x1p3|\n", [6]), "nanpay.tbl": (b"nan(12)|\n", [6]), "extra.tbl": (b"1|2|3|\n", [3, 3])}
    for name, (body, types) in bad.items():
        p = tmp_path / name
        p.write_bytes(body)
        codes = [ing.csv(str(p), types, [f"c{j}" for j in range(len(types))])[0] for _, ing in libs]
        assert codes[0] == codes[1] != 0, (name, codes)


def test_lineitem_1m_rows(libs, tmp_path):
    (gpu, ing), _ = libs
    text, exp = D.lineitem_csv(1_000_000, seed=5)
    p = tmp_path / "lineitem.tbl"
    p.write_bytes(text)
    rc, t = ing.csv(str(p), D.LINEITEM_TYPES, D.LINEITEM_NAMES)
    assert rc == 0, gpu.lib.hgpuLastError()
    names, cols = table_columns(gpu, t)
    assert names == D.LINEITEM_NAMES
    for name, col in zip(names, cols):
        e = exp[name]
        if name == "l_shipinstruct":
            assert col == [D._INSTRUCT[i] for i in e]
        elif name == "l_shipmode":
            assert col == [D._MODES[i] for i in e]
        elif name == "l_comment":
            assert col == e
        else:
            assert IC.same_column(col, e), name
    # the same table through the binary format, in HBM both ways
    b = str(tmp_path / "lineitem.bin")
    assert ing.save(b, t) == 0
    rc, t2 = ing.load(b)
    assert rc == 0
    IC.assert_same_table(table_columns(gpu, t2), (names, cols), "binary round trip")
    gpu.free_inputs()


def test_long_decimals_at_scale(libs, tmp_path):
    """Shortest round-trip texts of random doubles (up to 17 digits: mostly
    outside the fast path) and their float32 readings, against the oracle's
    strtod / strtof."""
    (gpu, ing), (ora, oing) = libs
    rng = np.random.default_rng(12)
    x = np.concatenate([rng.standard_normal(60_000) * 10.0 ** rng.integers(-300, 300, 60_000),
                        rng.random(20_000), np.exp(rng.uniform(-740, 709, 20_000))])
    lines = "".join(f"{repr(float(v))}|{repr(float(v))}|\n" for v in x)
    p = tmp_path / "doubles.tbl"
    p.write_text(lines)
    outs = []
    for lib, i in ((gpu, ing), (ora, oing)):
        rc, t = i.csv(str(p), [H_E, H_F], ["d", "f"])
        assert rc == 0
        outs.append(table_columns(lib, t)[1])
    assert IC.same_column(outs[0][0], x)
    assert IC.same_column(outs[0][1], outs[1][1])


def test_csv_host_residency(libs):
    (gpu, ing), _ = libs
    gpu.lib.hgpuSetResidency(1)
    try:
        case = IC.CSV_CASES[0]
        rc, t = ing.case(case)
        assert rc == 0
        vals = C.cast(t.g + 32, C.POINTER(C.c_uint8))  # the values node lives in host memory
        assert vals is not None
        IC.assert_same_table(table_columns(gpu, t), IC.load_table(EXPECT, case["id"]), "host residency")
    finally:
        gpu.lib.hgpuSetResidency(0)


def test_random_fields_match_oracle(libs, tmp_path):
    """Seeded random field texts (signs, spaces, tabs, junk suffixes, long
    digit runs, exponents, dates with signs and spaces) through every
    conversion, GPU against the oracle's strtol / strtod / strtof / sscanf."""
    rng = np.random.default_rng(31)
    n = 200_000

    def num_text(k):
        sign = ["", "+", "-", " -", "\t"][k % 5]
        digits = "".join(rng.choice(list("0123456789"), int(rng.integers(1, 25))))
        frac = "" if k % 3 else "." + "".join(rng.choice(list("0123456789"), int(rng.integers(0, 12))))
        exp = "" if k % 4 else f"e{int(rng.integers(-330, 330))}"
        tail = ["", "", "x", " 7", "e", "."][k % 6]
        return f"{sign}{digits}{frac}{exp}{tail}"

    def date_text(k):
        y, m, d = int(rng.integers(-3000, 3000)), int(rng.integers(-20, 40)), int(rng.integers(-5, 40))
        plus = lambda v: f"+{v}" if v >= 0 else f"{v}"  # noqa: E731  ("+-5" is not a %d)
        return [f"{y}-{m}-{d}", f" {y}- {m}- {d}", f"{plus(y)}-{plus(m)}-{d}junk", f"{y}-{m:02d}-{d:02d}"][k % 4]

    lines = []
    for k in range(n):
        t = num_text(k)
        lines.append(f"{t}|{t}|{t}|{t}|{t}|{t}|{t}|{date_text(k)}|{t[:1] or 'q'}|\n")
    p = tmp_path / "random.tbl"
    p.write_text("".join(lines))
    from horsepower_gb300.abi import H_B, H_C, H_D, H_F, H_H, H_I, H_J, H_L
    types = [H_E, H_F, H_L, H_I, H_J, H_H, H_B, H_D, H_C]
    outs = []
    for lib, ing in libs:
        rc, t = ing.csv(str(p), types, [f"c{j}" for j in range(len(types))])
        assert rc == 0
        outs.append(table_columns(lib, t)[1])
    for j, (a, b) in enumerate(zip(*outs)):
        assert IC.same_column(a, b), f"column {j}"
