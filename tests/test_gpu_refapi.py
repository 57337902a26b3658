"""The drop-in boundary for C++ callers: a program in the shape of the reference's main.cpp,
compiled against include/mhdgb_ref_api.hpp and linked with libmhdgb.so, reproduces the oracle bit
for bit (the header selects the separately rounded FP64 stage kernels)."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from mhdturbulence_gb300 import build, ic

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NX, NY, NZ, STEPS = 12, 16, 14, 6


def test_reference_shaped_program_matches_oracle(tmp_path):
    lib = build.build(driver=False)
    exe = str(tmp_path / "refapi_main")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "tests", "refapi"), os.path.join(ROOT, "tests", "refapi", "main.cpp"),
                    "-o", exe, "-L", os.path.dirname(lib), "-lmhdgb", f"-Wl,-rpath,{os.path.dirname(lib)}"],
                   check=True)
    out = str(tmp_path / "out.bin")
    subprocess.run([exe, out, str(STEPS)], check=True)
    it, jt, kt = ic.extents(NX, NY, NZ)
    N = it * jt * kt
    raw = np.fromfile(out, dtype=np.float64)
    P0 = raw[:12 * N].reshape(kt, jt, 12, it).copy()
    U0 = raw[12 * N:22 * N].reshape(kt, jt, 10, it).copy()
    U1 = raw[22 * N:32 * N].reshape(kt, jt, 10, it)
    P1 = raw[32 * N:44 * N].reshape(kt, jt, 12, it)
    dts = raw[44 * N:44 * N + STEPS]
    orc = O.Oracle(NX, NY, NZ, *ic.grid(NX, NY, NZ), gam=5.0 / 3.0, bc=ic.KH_BC, spacing_quirk=True)
    _, odts, _ = orc.run(U0, P0, STEPS)
    assert np.array_equal(dts, odts)
    assert np.array_equal(ic.interior(U1), ic.interior(U0))
    assert np.array_equal(ic.interior(P1), ic.interior(P0))


def test_cpp_driver_runs_kh_and_writes_tprof(tmp_path):
    build.build(driver=True)
    exe = os.path.join(os.path.dirname(build.LIB), "mhdgb_run")
    tp = str(tmp_path / "t-prof.csv")
    r = subprocess.run([exe, "-n", "24", "-t", "0.02", "-d", "10", "-o", tp], capture_output=True, text=True,
                       check=True)
    lines = r.stdout.splitlines()
    assert any(l.startswith("sim time [s]: ") for l in lines)
    tc = [l for l in lines if l.startswith("time/count/cell : ")]
    assert tc and float(tc[0].split(":")[1]) > 0
    rows = [l.split() for l in open(tp) if not l.startswith("#")]
    assert len(rows) >= 3 and all(len(x) == 4 for x in rows)
    t = [float(x[0]) for x in rows]
    assert t[0] == 0.0 and t[-1] > 0.02 and all(b >= a for a, b in zip(t, t[1:]))
