"""Generate the golden vectors in this folder by running the reference's own solver stages and its
own output routine.

The reference's src_cpp_kokkos_host/{mhd,boundary,mpi_config}.cpp are compiled unmodified from the
reference tree against oracle/refshim/ (``make -C oracle ref``), driven by oracle/refshim/ref_harness.cpp
in the stage order of src_cpp_kokkos_host/main.cpp:229-259, and their outputs are stored here as
compressed .npz files.  Needs the reference tree (only present where the fixtures are made);
the tests only read the .npz files.

    python tests/golden/make_golden.py [--refdir /path/to/src_cpp_kokkos_host] [--only stages|output]

Each case stores:  meta (nx,ny,nz,gam,bc,nsteps,domain), U0 (input conserved state; only the
interior is meaningful), dts/chgs (per step), and interior or full arrays P0 (UpdatePrimitvP of
the input), P1/U1 (after step 1), PN/UN (after nsteps), F1 (the three face-flux arrays of step 1,
full cases only).

The output case (output_7x5x4.npz) runs the reference's Output() (src_cpp_kokkos_host/output.cpp,
``make -C oracle refout``, driven by oracle/refshim/ref_output.cpp) on two primitive states and
stores: meta (nx,ny,nz), domain, td (time, dt per snapshot), P (the full input arrays) and every
file it wrote (names: relative paths, blob_<i>: the bytes).
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mhdturbulence_gb300 import ic  # noqa: E402

CASES = [
    # name, (nx,ny,nz), prim-builder, domain, bc, nsteps, full
    ("kh_6x8x7", (6, 8, 7), lambda n: ic.kh_prim(*n, seed=11, amp=0.05, noise=1e-2), ic.KH_DOMAIN,
     ic.KH_BC, 5, True),
    ("mixedbc_5x7x9", (5, 7, 9), lambda n: ic.random_smooth_prim(*n, seed=5), ic.CUBE_DOMAIN,
     (ic.BC_OUTFLOW, ic.BC_REFLECTION, ic.BC_PERIODIC, ic.BC_PERIODIC, ic.BC_REFLECTION, ic.BC_OUTFLOW), 6, False),
    ("refkh_noB_8x8x8", (8, 8, 8), lambda n: ic.ref_kh_prim(*n), ic.KH_DOMAIN, ic.KH_BC, 10, False),
    ("turb_8x8x8", (8, 8, 8), lambda n: ic.turbulence_prim(8, seed=9), ic.CUBE_DOMAIN, ic.PERIODIC_BC, 10, False),
]
GAM = 5.0 / 3.0


def domain_flags(domain) -> str:
    (a, b), (c, d), (e, f) = domain
    vals = dict(X1MIN=a, X1MAX=b, X2MIN=c, X2MAX=d, X3MIN=e, X3MAX=f)
    return " ".join(f"'-DREF_{k}=({v!r})'" for k, v in vals.items())


def build_ref(n, domain, refdir, tag):
    nx, ny, nz = n
    exe = os.path.join(ROOT, "oracle", "_ref", f"ref_{nx}x{ny}x{nz}")
    # one binary per (grid, domain): build into a unique name
    exe_tag = exe + "_" + tag
    subprocess.run(["make", "-s", "-B", "-C", os.path.join(ROOT, "oracle"), "ref",
                    f"NX={nx}", f"NY={ny}", f"NZ={nz}", f"REFDIR={refdir}",
                    f"DOMAIN={domain_flags(domain)}"], check=True)
    os.replace(exe, exe_tag)
    return exe_tag


def run_ref(exe, n, U0, bc, nsteps, dump_flux):
    nx, ny, nz = n
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([nx, ny, nz], dtype="<i4").tofile(f)
            np.array([GAM], dtype="<f8").tofile(f)
            np.array(bc, dtype="<i4").tofile(f)
            np.array([nsteps, 1 if dump_flux else 0], dtype="<i4").tofile(f)
            U0.astype("<f8").tofile(f)
        subprocess.run([exe, fin, fout], check=True, env=dict(os.environ, OMP_NUM_THREADS="2"))
        raw = np.fromfile(fout, dtype="<f8")
    it, jt, kt = ic.extents(nx, ny, nz)
    N = it * jt * kt
    off = 0

    def take(cnt):
        nonlocal off
        a = raw[off:off + cnt]
        off += cnt
        return a

    out = {"dts": take(nsteps), "chgs": take(nsteps)}
    shp = lambda nv: (kt, jt, nv, it)  # noqa: E731
    out["P0"] = take(12 * N).reshape(shp(12))
    out["P1"] = take(12 * N).reshape(shp(12))
    out["U1"] = take(10 * N).reshape(shp(10))
    if dump_flux:
        out["F1"] = take(30 * N).reshape((3,) + shp(10))
    out["PN"] = take(12 * N).reshape(shp(12))
    out["UN"] = take(10 * N).reshape(shp(10))
    assert off == raw.size
    return out


OUTPUT_CASE = ("output_7x5x4", (7, 5, 4), ic.KH_DOMAIN, [(0.0, 0.0), (0.12345678901234567, 1.5e-3)])


def make_output_golden(refdir):
    name, (nx, ny, nz), domain, td = OUTPUT_CASE
    subprocess.run(["make", "-s", "-B", "-C", os.path.join(ROOT, "oracle"), "refout", f"NX={nx}", f"NY={ny}",
                    f"NZ={nz}", f"REFDIR={refdir}", f"DOMAIN={domain_flags(domain)}"], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", f"refout_{nx}x{ny}x{nz}")
    it, jt, kt = ic.extents(nx, ny, nz)
    rng = np.random.default_rng(77)
    Ps = np.stack([rng.uniform(0.5, 2.0, (kt, jt, 12, it)), rng.standard_normal((kt, jt, 12, it))])
    with tempfile.TemporaryDirectory() as tdir:
        fin = os.path.join(tdir, "in.bin")
        with open(fin, "wb") as f:
            np.array([nx, ny, nz, len(td)], dtype="<i4").tofile(f)
            for (t, dt), P in zip(td, Ps):
                np.array([t, dt], dtype="<f8").tofile(f)
                P.astype("<f8").tofile(f)
        subprocess.run([exe, fin], check=True, cwd=tdir, stdout=subprocess.DEVNULL)
        names = sorted(os.path.relpath(os.path.join(d, fn), tdir) for d, _, fs in os.walk(tdir) for fn in fs
                       if fn != "in.bin")
        blobs = {f"blob_{i}": np.frombuffer(open(os.path.join(tdir, nm), "rb").read(), dtype=np.uint8)
                 for i, nm in enumerate(names)}
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, meta=np.array([nx, ny, nz]), domain=np.array(domain, dtype=np.float64),
                        td=np.array(td, dtype=np.float64), P=Ps, names=np.array(names), **blobs)
    print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB, files: {' '.join(names)}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--refdir", default=os.environ.get("MHDTURB_REFDIR"), required="MHDTURB_REFDIR" not in os.environ,
                    help="the reference's src_cpp_kokkos_host directory (or set MHDTURB_REFDIR)")
    ap.add_argument("--only", choices=["stages", "output"], default=None)
    args = ap.parse_args()
    if args.only != "stages":
        make_output_golden(args.refdir)
    if args.only == "output":
        return
    for name, n, builder, domain, bc, nsteps, full in CASES:
        exe = build_ref(n, domain, args.refdir, name)
        U0 = ic.prim_to_cons(builder(n), GAM)
        res = run_ref(exe, n, U0, bc, nsteps, dump_flux=full)
        meta = np.array([*n, nsteps, *bc], dtype=np.int64)
        store = {"meta": meta, "gam": np.array([GAM]), "domain": np.array(domain, dtype=np.float64),
                 "dts": res["dts"], "chgs": res["chgs"], "U0": ic.interior(U0).copy()}
        for key in ("P0", "P1", "U1", "PN", "UN"):
            store[key] = res[key] if full else ic.interior(res[key]).copy()
        if full:
            store["F1"] = res["F1"]
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **store)
        print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB, dt0={res['dts'][0]:.6e}, chg0={res['chgs'][0]:.6e}")


if __name__ == "__main__":
    main()
