"""Snapshot output on the GPU path (mhdgb_output*) against the files the reference's own Output()
wrote for the same states (tests/golden/output_7x5x4.npz), byte for byte, and the asynchronous form
against the synchronous one while later steps run."""
import os
import sys

import numpy as np
import pytest

from mhdturbulence_gb300 import MhdgbError, Solver, ic

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import output_oracle  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(HERE, "golden", "output_7x5x4.npz")


def read_tree(root):
    return {os.path.relpath(os.path.join(d, f), root): open(os.path.join(d, f), "rb").read()
            for d, _, fs in os.walk(root) for f in fs}


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64", "mixed"])
def test_output_files_equal_the_reference_files(tmp_path, precision):
    z = np.load(GOLDEN)
    want = {str(n): z[f"blob_{i}"].tobytes() for i, n in enumerate(z["names"])}
    nx, ny, nz = (int(v) for v in z["meta"])
    domain = tuple(map(tuple, z["domain"]))
    with Solver(nx, ny, nz, domain=domain, precision=precision) as s:
        for index, ((t, dt), P) in enumerate(zip(z["td"], z["P"])):
            s.upload_prim(P)
            s.output(str(tmp_path), index, float(t), float(dt), ascii=True)
    got = read_tree(tmp_path)
    assert sorted(got) == sorted(want)
    for name in want:
        assert got[name] == want[name], name


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_async_output_is_the_state_at_begin(tmp_path, precision):
    nx, ny, nz = 24, 16, 12
    with Solver(nx, ny, nz, precision=precision) as s:
        s.init_kh(seed=4)
        s.step(5)
        r = s.sync()
        s.output_begin(str(tmp_path / "a"), 3, r.time, r.dt, ascii=True)
        s.step(7)                                  # overlaps the copy and the writer
        s.output_end()
        r2 = s.sync()
        assert r2.step == 12
    with Solver(nx, ny, nz, precision=precision) as s:
        s.init_kh(seed=4)
        s.step(5)
        r = s.sync()
        P5 = s.download_prim()
        axes = s.grid()
        s.output(str(tmp_path / "b"), 3, r.time, r.dt, ascii=True)
    a, b = read_tree(tmp_path / "a"), read_tree(tmp_path / "b")
    assert a == b
    field = np.frombuffer(a["bindata/field00003.bin"], dtype="<f8").reshape(10, nz, ny, nx)
    assert np.array_equal(field, output_oracle.pack(P5, nx, ny, nz))
    output_oracle.write_output(str(tmp_path / "c"), 3, P5, axes, r.time, r.dt)
    assert read_tree(tmp_path / "c") == a


def test_unwritable_root_reports_io_error(tmp_path):
    (tmp_path / "file").write_text("x")
    with Solver(8, 8, 8) as s:
        s.init_kh()
        with pytest.raises(MhdgbError) as e:
            s.output(str(tmp_path / "file" / "sub"), 0, 0.0, 0.0)
        assert e.value.code == -9
        s.output(str(tmp_path / "ok"), 0, 0.0, 0.0)        # the handle stays usable
    assert os.path.exists(tmp_path / "ok" / "bindata" / "field00000.bin")
