"""The oracle's restatement of the reference's table loaders (readCSV,
serializeV / readSerializeV, h_io.cc) against the reference's own results on
the ingest fixtures (CPU suite)."""
import os

import numpy as np
import pytest

import ingest_cases as IC
from ingest_run import FIXTURES, Ingest
from horsepower_gb300.abi import Builtins, table_columns

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXPECT = np.load(os.path.join(ROOT, "tests", "golden", "ingest.npz"))


@pytest.fixture(scope="module")
def ora():
    import subprocess
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    lib = Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")
    return lib, Ingest(lib)


@pytest.mark.parametrize("case", IC.CSV_CASES, ids=[c["id"] for c in IC.CSV_CASES])
def test_oracle_csv_matches_reference(ora, case):
    lib, ing = ora
    rc, t = ing.case(case)
    assert rc == 0
    IC.assert_same_table(table_columns(lib, t), IC.load_table(EXPECT, case["id"]), case["id"])


def test_oracle_reads_reference_binaries(ora, tmp_path):
    lib, ing = ora
    rc, t = ing.load(os.path.join(FIXTURES, "lineitem_1k.bin"))
    assert rc == 0
    IC.assert_same_table(table_columns(lib, t), IC.load_table(EXPECT, "lineitem"), "lineitem.bin")
    rc, v = ing.load(os.path.join(FIXTURES, "vectors.bin"))
    assert rc == 0
    IC.assert_same_node(IC.node_to_py(lib, v), IC.load_vectors(EXPECT, "vectors"))
    # write and read back
    p = str(tmp_path / "t.bin")
    assert ing.save(p, t) == 0
    rc, t2 = ing.load(p)
    assert rc == 0
    IC.assert_same_table(table_columns(lib, t2), IC.load_table(EXPECT, "lineitem"), "round trip")


def test_oracle_csv_errors(ora, tmp_path):
    lib, ing = ora
    bad = {"fields.tbl": (b"1|2|\n3|\n", [3, 3], 2), "long.tbl": (b"1|" + b"7" * 1100 + b"|\n", [3, 3], 2),
           "nul.tbl": (b"1|2\x003|\n", [3, 3], 2), "date.tbl": (b"1994/01/01|\n", [12], 2),
           "hex.tbl": (b"0x1p3|\n", [6], 99), "nanpay.tbl": (b"nan(12)|\n", [6], 99)}
    for name, (body, types, code) in bad.items():
        p = tmp_path / name
        p.write_bytes(body)
        rc, _ = ing.csv(str(p), types, [f"c{j}" for j in range(len(types))])
        assert rc == code, name
