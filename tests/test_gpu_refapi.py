"""The drop-in boundary for C++ callers: a program in the shape of the reference's main.cpp,
compiled against include/mhdgb_ref_api.hpp and linked with libmhdgb.so, reproduces the oracle bit
for bit (the header selects the separately rounded FP64 stage kernels), and its forced Output()
calls write the reference's snapshot files."""
import os
import subprocess
import sys

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
    run_dir = tmp_path / "run"
    run_dir.mkdir()
    subprocess.run([exe, out, str(STEPS)], check=True, cwd=run_dir)
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
    # the two forced snapshots: the uploaded initial P at t = 0 (dt not yet set: 0), the final P
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import output_oracle
    axes = ic.grid(NX, NY, NZ)
    P_init = raw[:12 * N].reshape(kt, jt, 12, it)
    output_oracle.write_output(str(tmp_path / "want"), 0, P_init, axes, 0.0, 0.0)
    t_end = 0.0
    for d in dts:                                   # time_sim += dt, in step order
        t_end += float(d)
    output_oracle.write_output(str(tmp_path / "want"), 1, P1, axes, t_end, float(dts[-1]))

    def tree(root):
        return {os.path.relpath(os.path.join(d, f), root): open(os.path.join(d, f), "rb").read()
                for d, _, fs in os.walk(root) for f in fs}
    got, want = tree(run_dir), tree(tmp_path / "want")
    assert sorted(got) == sorted(want)
    for name in want:
        assert got[name] == want[name], name


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


def test_cpp_driver_writes_reference_snapshots(tmp_path):
    """--output/--dtout: forced snapshots at the start and the end, regular ones each time the time
    reaches the previous snapshot's + dtout (main.cpp:219, 261, 279); the last one is the state a
    Python-side run of the same problem reaches."""
    from mhdturbulence_gb300 import Solver
    build.build(driver=True)
    exe = os.path.join(os.path.dirname(build.LIB), "mhdgb_run")
    out = tmp_path / "snap"
    n, tmax, dtout = 16, 0.05, 0.02
    r = subprocess.run([exe, "-n", str(n), "-t", str(tmax), "--output", str(out), "--dtout", str(dtout), "--ascii",
                        "-o", str(tmp_path / "t-prof.csv")], capture_output=True, text=True, check=True)
    idx = [l for l in r.stdout.splitlines() if l.startswith("output index=")]
    times = []
    for i in range(len(idx)):
        head = open(out / "bindata" / f"unf{i:05d}.dat").read().split("\n")[0].split()
        times.append(float(head[1]))
        assert (out / "bindata" / f"field{i:05d}.bin").stat().st_size == 10 * n ** 3 * 8
        assert (out / "ascdata" / f"snap000-{i:05d}.csv").exists()
    assert len(times) >= 4 and times[0] == 0.0
    assert all(b >= a + dtout for a, b in zip(times[:-2], times[1:-1]))   # regular snapshots
    assert times[-1] > tmax and times[-1] >= times[-2]                   # the forced final snapshot
    with Solver(n, n, n, precision="fp64") as s:
        s.init_kh(seed=1)
        rep = s.run_until(tmax)
        P = s.download_prim()
        assert rep.time == times[-1]
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import output_oracle
    got = np.fromfile(out / "bindata" / f"field{len(times) - 1:05d}.bin", dtype="<f8")
    assert np.array_equal(got, output_oracle.pack(P, n, n, n).ravel())


def test_cpp_driver_restart_equals_uninterrupted_run(tmp_path):
    """--checkpoint / --restart: a run to t = 0.02 restarted to t = 0.04 ends in the same state and
    clock, byte for byte in the checkpoint file, as one run to t = 0.04."""
    build.build(driver=True)
    exe = os.path.join(os.path.dirname(build.LIB), "mhdgb_run")
    common = ["-n", "16", "-p", "fp64", "-o", str(tmp_path / "t.csv")]
    a, b, c = (str(tmp_path / f) for f in ("a.ck", "b.ck", "c.ck"))
    subprocess.run([exe, *common, "-t", "0.02", "--checkpoint", a], check=True, capture_output=True)
    subprocess.run([exe, *common, "-t", "0.04", "--restart", a, "--checkpoint", b], check=True, capture_output=True)
    subprocess.run([exe, *common, "-t", "0.04", "--checkpoint", c], check=True, capture_output=True)
    assert open(b, "rb").read() == open(c, "rb").read()
    assert open(a, "rb").read() != open(c, "rb").read()
