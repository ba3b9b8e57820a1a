"""Solution output in the crate's CSV format (Solution::to_csv, src/solution.rs:190-226): header
t,y0,...,yN-1, numbers formatted like Rust's `{:?}` for f64.  Python (degpu.write_csv) and C++
(degpu.hpp Solution::to_csv) writers are checked against the same expectations."""
import os
import subprocess

import numpy as np
import pytest

import degpu
from degpu import rust_debug_f64

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KNOWN = [(1.0, "1.0"), (0.1, "0.1"), (1e-4, "0.0001"), (1e-5, "1e-5"), (1.5e16, "1.5e16"), (1e16, "1e16"),
         (9999999999999998.0, "9999999999999998.0"), (-0.0, "-0.0"), (0.0, "0.0"), (2.5e-300, "2.5e-300"),
         (float("nan"), "NaN"), (float("inf"), "inf"), (float("-inf"), "-inf"), (123.456, "123.456"),
         (-3e-7, "-3e-7"), (1e15, "1000000000000000.0"), (22026.465794806718, "22026.465794806718")]


def test_rust_debug_format_known_values():
    for v, s in KNOWN:
        assert rust_debug_f64(v) == s, (v, rust_debug_f64(v), s)


def test_write_csv(tmp_path):
    p = tmp_path / "sub" / "sol.csv"
    degpu.write_csv(str(p), [0.0, 0.5], [[1.0, -2.5], [1e16, 0.1]])
    assert p.read_text() == "t,y0,y1\n0.0,1.0,-2.5\n0.5,1e16,0.1\n"


def test_cpp_writer_matches(tmp_path):
    exe = tmp_path / "csvcheck"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"),
                        os.path.join(REPO, "tests", "cpp", "csv_format_check.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("C++17 compiler without floating-point to_chars: " + r.stderr[-200:])
    rng = np.random.default_rng(21)
    vals = [v for v, _ in KNOWN] + list(rng.standard_normal(2000) * 10.0 ** rng.integers(-30, 30, 2000))
    inp = "\n".join(float(v).hex() if np.isfinite(v) else repr(float(v)) for v in vals) + "\n"
    csv = tmp_path / "d" / "cpp.csv"
    out = subprocess.run([str(exe), str(csv)], input=inp, capture_output=True, text=True, check=True).stdout.split()
    assert out == [rust_debug_f64(v) for v in vals]
    assert csv.read_text() == "t,y0,y1\n0.0,1.0,-2.5\n0.5,1e16,0.1\n1e-5,2.5e-300,-0.0\n"
