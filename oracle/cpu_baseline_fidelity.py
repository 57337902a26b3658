"""Speed of the oracle port against the reference's own CPU stages, on the same cores and input.

TEST INFRASTRUCTURE.  The timed CPU baseline on the GPU host is the oracle port (oracle/mhd_oracle.c):
the reference's sources cannot travel there.  This script measures how far the port's speed is from
the reference's own src_cpp_kokkos_host stages (compiled unmodified against oracle/refshim, `make ref`)
where both can run: it builds the reference at the grid, steps the KH state `--steps` times with
each on `--threads` OpenMP threads, prints both `time/count/cell` figures (the reference's report,
main.cpp:274-276) and their ratio, and checks that the two final states are equal bit for bit.

    MHDTURB_REFDIR=<reference>/src_cpp_kokkos_host python oracle/cpu_baseline_fidelity.py --n 150
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402
from mhdturbulence_gb300 import ic  # noqa: E402

GAM = 5.0 / 3.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--refdir", default=os.environ.get("MHDTURB_REFDIR"), required="MHDTURB_REFDIR" not in os.environ)
    ap.add_argument("--n", type=int, default=150)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--repeats", type=int, default=3)
    args = ap.parse_args()
    n = args.n
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"NX={n}", f"NY={n}", f"NZ={n}", f"REFDIR={args.refdir}"],
                   check=True)
    exe = os.path.join(HERE, "_ref", f"ref_{n}x{n}x{n}")
    U0 = ic.prim_to_cons(ic.kh_prim(n, n, n, seed=1), GAM)
    env = dict(os.environ, OMP_NUM_THREADS=str(args.threads), OMP_PROC_BIND="close")

    ref_s, ref_U = [], None
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([n, n, n], dtype="<i4").tofile(f)
            np.array([GAM], dtype="<f8").tofile(f)
            np.array(ic.KH_BC, dtype="<i4").tofile(f)
            np.array([args.steps, 0], dtype="<i4").tofile(f)
            U0.astype("<f8").tofile(f)
        for _ in range(args.repeats):
            r = subprocess.run([exe, fin, fout], check=True, env=env, capture_output=True, text=True)
            ref_s.append(float(re.search(r"time/count/cell : (\S+)", r.stderr).group(1)))
        raw = np.fromfile(fout, dtype="<f8")
        ref_U = raw[-U0.size:].reshape(U0.shape)

    O.set_threads(args.threads)
    orc = O.Oracle(n, n, n, *ic.grid(n, n, n, ic.KH_DOMAIN), gam=GAM, bc=ic.KH_BC, spacing_quirk=True)
    port_s, port_U = [], None
    for _ in range(args.repeats):
        U, P = U0.copy(), ic.empty_field(n, n, n, 12)
        orc.update_prim(U, P)
        t0 = time.perf_counter()
        orc.run(U, P, args.steps)
        port_s.append((time.perf_counter() - t0) / n ** 3 / args.steps)
        port_U = U
    ref_best, port_best = min(ref_s), min(port_s)
    same = bool(np.array_equal(ic.interior(ref_U), ic.interior(port_U)))
    print(f"KH {n}^3, {args.steps} steps, {args.threads} threads (best of {args.repeats})")
    print(f"reference (src_cpp_kokkos_host stages on refshim): time/count/cell : {ref_best:e}"
          f"  ({1e-9 / ref_best:.5f} Gcell-updates/s)")
    print(f"oracle port (mhd_oracle.c):                         time/count/cell : {port_best:e}"
          f"  ({1e-9 / port_best:.5f} Gcell-updates/s)")
    print(f"port speed / reference speed = {ref_best / port_best:.3f}; final states equal bit for bit: {same}")


if __name__ == "__main__":
    main()
