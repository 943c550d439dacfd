"""The native CSV reader (gwgpu_csv_read): no GPU involved.  It must give the
exact doubles Python writes with repr, accept the forms Armadillo's csv_name
files take (quoted or bare header, CRLF, blank lines), and reject malformed
cells with the line number."""
import json
import os

import numpy as np
import pytest

from libgwmodel_gb300 import GwgpuError
from libgwmodel_gb300.io import read_csv

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write(path, text):
    with open(path, "w", newline="") as f:
        f.write(text)
    return path


def test_londonhp100_round_trip(tmp_path):
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "londonhp100.json")))
    data = np.array(g["data"])
    lines = ['"PURCHASE","FLOORSZ","UNEMPLOY","PROF"'] + [",".join(repr(float(v)) for v in row) for row in data]
    t = read_csv(write(tmp_path / "d.csv", "\n".join(lines) + "\n"))
    assert t.names == ["PURCHASE", "FLOORSZ", "UNEMPLOY", "PROF"]
    assert (t.rows, t.cols) == (100, 4)
    np.testing.assert_array_equal(t.columns(), data)
    np.testing.assert_array_equal(t.columns(["PROF", "FLOORSZ"]), data[:, [3, 1]])
    np.testing.assert_array_equal(t.column("PURCHASE"), data[:, 0])
    assert t.columns(["PROF"]).flags.f_contiguous


def test_forms(tmp_path):
    t = read_csv(write(tmp_path / "a.csv", "x, y\r\n1, 2.5\r\n\r\n-3e2,+4\r\n  \n5 ,6"))
    assert t.names == ["x", "y"]
    np.testing.assert_array_equal(t.columns(), [[1, 2.5], [-300, 4], [5, 6]])


def test_parallel_parse_matches_numpy(tmp_path):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((100_003, 5)) * 10.0 ** rng.integers(-8, 8, (100_003, 5))
    path = tmp_path / "big.csv"
    with open(path, "w") as f:
        f.write("a,b,c,d,e\n")
        for row in a:
            f.write(",".join(repr(float(v)) for v in row) + "\n")
    t = read_csv(path)
    np.testing.assert_array_equal(t.columns(), a)


@pytest.mark.parametrize("body, line, what", [
    ("x,y\n1,2\n3,\n", 3, "empty cell"),
    ("x,y\n1,2\n3,abc\n", 3, "not a number"),
    ("x,y\n1,2\n3\n", 3, "expected 2 cells"),
    ("x,y\n1,2,3\n", 2, "more than 2 cells"),
])
def test_errors_name_the_line(tmp_path, body, line, what):
    with pytest.raises(GwgpuError) as e:
        read_csv(write(tmp_path / "bad.csv", body))
    assert f":{line}: " in str(e.value) and what in str(e.value)


def test_unknown_column_and_missing_file(tmp_path):
    t = read_csv(write(tmp_path / "a.csv", "x,y\n1,2\n"))
    with pytest.raises(GwgpuError):
        t.columns(["z"])
    with pytest.raises(GwgpuError):
        read_csv(tmp_path / "missing.csv")
