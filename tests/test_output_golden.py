"""The output oracle (oracle/output_oracle.py) against the files the reference's own Output()
wrote (tests/golden/output_7x5x4.npz, made by tests/golden/make_golden.py): byte for byte."""
import os
import sys

import numpy as np
import pytest

from mhdturbulence_gb300 import ic

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import output_oracle  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "output_7x5x4.npz")


def golden_files():
    z = np.load(GOLDEN)
    return z, {str(n): z[f"blob_{i}"].tobytes() for i, n in enumerate(z["names"])}


def test_output_oracle_matches_reference_files(tmp_path):
    z, want = golden_files()
    nx, ny, nz = (int(v) for v in z["meta"])
    axes = ic.grid(nx, ny, nz, tuple(map(tuple, z["domain"])))
    for index, ((t, dt), P) in enumerate(zip(z["td"], z["P"])):
        output_oracle.write_output(str(tmp_path), index, P, axes, float(t), float(dt))
    got = {os.path.relpath(os.path.join(d, f), tmp_path): open(os.path.join(d, f), "rb").read()
           for d, _, fs in os.walk(tmp_path) for f in fs}
    assert sorted(got) == sorted(want)
    for name in want:
        assert got[name] == want[name], name


def test_golden_field_file_is_the_packed_state():
    z, want = golden_files()
    nx, ny, nz = (int(v) for v in z["meta"])
    data = np.frombuffer(want["bindata/field00001.bin"], dtype="<f8").reshape(10, nz, ny, nx)
    assert np.array_equal(data, output_oracle.pack(z["P"][1], nx, ny, nz))
    assert data[0, 0, 0, 0] == z["P"][1][2, 2, 0, 2]
    assert data[8, 0, 0, 0] == z["P"][1][2, 2, 5, 2]   # p is written after bp
