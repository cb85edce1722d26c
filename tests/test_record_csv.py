"""The CSV export (Settings::save_data, src/settings.rs:2014-2052) writes the
reference's header and prints every number as the reference does (Rust's
Display of f64): the first lines of the reference's own TEXP_1.csv, read as
numbers and written back, give the same text byte for byte."""
import os

import numpy as np

import record


def test_csv_text_equals_the_reference_export(golden_dir, tmp_path):
    src = os.path.join(golden_dir, "TEXP_1_head.csv")
    text = open(src).read()
    rows = np.loadtxt(src, delimiter=",", skiprows=1, dtype=np.float64, ndmin=2)
    out = tmp_path / "out.csv"
    record.write_csv(str(out), rows[:, :11], fps=rows[:, 11])
    assert open(out).read() == text


def test_number_format_is_positional_shortest_round_trip():
    for x in (0.0, -0.0, 1.0, 24.99500274658203, 4.9990007688904825e-09, 1e-20, 1e21, -3.25):
        s = record.format_f64(x)
        assert "e" not in s and float(s) == x
    assert record.format_f64(0.0) == "0" and record.format_f64(25.0) == "25"
