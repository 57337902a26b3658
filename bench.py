#!/usr/bin/env python3
"""Benchmark of the MHDTurbulence solver step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--grid 150]

Workload: the reference's benchmark problem, Kelvin-Helmholtz on 150^3 cells (x in [-0.5,0.5],
y in [-1,1], z in [-0.5,0.5]; periodic x/z, reflecting y), gamma = 5/3, dt = 0.05 * CFL minimum,
FP64 form; one "step" is one full solver step (dt/c_h reductions, ghost fill, x/y/z HLLD fluxes
with GLM, update, psi damping, primitive recovery).  Seeded synthetic initial data (the KH set-up
of mhdturbulence_gb300/ic.py, generated on the device by mhdgb_init_kh).

Prints one JSON line.  value = whole-job Gcell-updates/s of the FP64 form with the state resident
in HBM (CUDA events on the launching stream, W warm-up steps, then K timed steps; the 150^3 state
is ~1 GB, larger than L2, so no flush is needed); e2e = the same through mhdgb_step_host with the
state in pinned host memory, moved in and out every step (298 MB each way over the host link);
"mixed" = the FP32-mixed form on the same configuration, with its own e2e and its error against
the FP64 form; "size_256" = both forms on KH 256^3 (the size the FP64-roofline and mixed-speed-up
targets are quoted at); "ensemble" = 64 seeded uneven KH grids in one persistent launch per step,
mixed and FP64, against one 512^3 mixed grid; cpu_baseline = the oracle (the reference's
arithmetic restated in C, OpenMP) on this host's cores.

--impl reference times the reference's CPU path on the host cores: the reference sources cannot
be built on this machine (they need Kokkos and MPI, and the reference tree is absent here), so the
oracle port stands in for it, with all host threads.  On the same cores (KH 150^3, 8 threads, best of
3 runs of 6 steps) the port runs 1.08x as fast as the reference's own stages built against a
Kokkos/MPI shim, with equal final states (oracle/cpu_baseline_fidelity.py), so the ratio against this
arm understates the speed-up over the reference itself by about that factor.

Multi-GPU (torchrun): the ranks hold the 150^3 blocks of one 150 x 150 x (150 N) KH grid split
along z and swap the halos of their shared faces over NCCL after every step, with dt and c_h
all-reduced (mhdturbulence_gb300.distributed; weak scaling); timings are max-reduced over ranks,
value sums all ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ns/cell/step & Gcell-updates/s on 1 GB300: FP32-mixed vs FP64 at stated error"
B_ALG = 160  # bytes per cell-update: 10 FP64 conserved fields read once and written once
# published 4xA100 figure for the same problem (f90 OpenACC, reference README.md:95), for context
PUBLISHED_4XA100_S_PER_CELL_STEP = 1.14e-9


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_summary(name):
    """Per-cell DRAM bytes / FP64 instruction counts of a kernel from a committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            return json.load(f)
    except Exception:
        return None


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        for line in (getattr(self, "out", "") or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 8:
                rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][1]) if rows[0][1].replace(".", "").isdigit() else None,
                "power_w_max": max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit()),
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ws, cells_per_rank, steps, ms_max):
    """Whole-job Gcell-updates/s of ws independent replicas: the cells all ranks updated over the
    slowest rank's time (weak scaling, no data exchange between ranks)."""
    return ws * cells_per_rank * steps / (ms_max * 1e-3) / 1e9


def cpu_oracle_rate(n, max_seconds, warm=1, max_steps=None):
    """Gcell-updates/s of the oracle on KH n^3 with all host threads; bounded wall time."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from mhdturbulence_gb300 import ic

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    gam = 5.0 / 3.0
    U = ic.prim_to_cons(ic.kh_prim(n, n, n, seed=1), gam)
    P = ic.empty_field(n, n, n, 12)
    orc = O.Oracle(n, n, n, *ic.grid(n, n, n), gam=gam, bc=ic.KH_BC, spacing_quirk=False)
    orc.update_prim(U, P)
    orc.run(U, P, warm)
    t0 = time.perf_counter()
    steps = 0
    while True:
        orc.run(U, P, 1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= max_seconds or (max_steps is not None and steps >= max_steps):
            break
    return n ** 3 * steps / el / 1e9, threads, steps, el


def run_reference(args, ws, rank):
    if rank != 0:
        return
    rate, threads, steps, el = cpu_oracle_rate(args.n, args.cpu_seconds_ref, warm=max(1, min(args.warmup, 2)),
                                               max_steps=args.steps)
    sample = (f"KH {args.n}^3 FP64, {steps} full steps after warm-up, {el:.1f} s wall, OMP threads={threads} "
              "(oracle port of src_cpp_kokkos_host: the reference's own build needs Kokkos and MPI, which "
              "this host lacks, and its sources do not travel to the GPU host)")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "Gcell-updates/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": el / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "ns_per_cell_step": 1.0 / rate,
        "config": bench_config(args.n, ws),
        "cpu_baseline": {"value": rate, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": rate, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def mixed_error(n, steps, device):
    """Error of the mixed form against the FP64 form after `steps` steps from the same state."""
    from mhdturbulence_gb300 import Solver, ic
    out = {}
    for prec in ("fp64", "mixed"):
        with Solver(n, n, n, precision=prec, device=device) as s:
            s.init_kh(seed=1)
            s.step(steps)
            r = s.sync()
            U = ic.interior(s.download_cons())
            P = ic.interior(s.download_prim())
            x1a, x2a, x3a = s.grid()
            out[prec] = (r, U, P, (x1a, x2a, x3a))
    (rd, Ud, Pd, g), (rm, Um, Pm, _) = out["fp64"], out["mixed"]
    rho_d, rho_m = Ud[:, :, 0, :], Um[:, :, 0, :]

    def divb(P):
        dx = np.diff(g[0])[2:2 + n]
        dy = np.diff(g[1])[2:2 + n]
        dz = np.diff(g[2])[2:2 + n]
        bx, by, bz = P[:, :, 7, :], P[:, :, 8, :], P[:, :, 9, :]
        d = (np.roll(bx, -1, 2) - np.roll(bx, 1, 2)) / (2 * dx[None, None, :]) \
            + (np.roll(by, -1, 1) - np.roll(by, 1, 1)) / (2 * dy[None, :, None]) \
            + (np.roll(bz, -1, 0) - np.roll(bz, 1, 0)) / (2 * dz[:, None, None])
        return float(np.sqrt(np.mean(d[:, 1:-1, :] ** 2)))

    return {
        "steps": steps,
        "rho_l1_rel": float(np.abs(rho_m - rho_d).sum() / np.abs(rho_d).sum()),
        "rho_linf_rel": float(np.abs(rho_m - rho_d).max() / np.abs(rho_d).max()),
        "energy_l1_rel": float(np.abs(Um[:, :, 4, :] - Ud[:, :, 4, :]).sum() / np.abs(Ud[:, :, 4, :]).sum()),
        "total_energy_rel": float(abs(Um[:, :, 4, :].sum() / Ud[:, :, 4, :].sum() - 1)),
        "divB_rms_fp64": divb(Pd), "divB_rms_mixed": divb(Pm),
        "time_rel": float(abs(rm.time / rd.time - 1)),
    }


def run_only(args, local):
    """Lean run of one form (no autotune, e2e, CPU or error legs): the target of kernel profiles."""
    from mhdturbulence_gb300 import Solver
    n = args.n
    with Solver(n, n, n, precision=args.only, device=local) as s:
        s.select_variant(args.variant)
        s.init_kh(seed=1)
        s.time_steps(args.warmup)
        ms = s.time_steps(args.steps)
        r = s.sync()
        tx, ty, nt, _ = s.variants()[args.variant]
    print(json.dumps({"form": args.only, "n": n, "tile": f"{tx}x{ty}/{nt}", "steps": args.steps,
                      "ms_per_step": ms / args.steps, "ns_per_cell_step": ms / args.steps * 1e6 / n ** 3,
                      "status": int(r.status)}), flush=True)


def bench_config(n, ws):
    """The workload description both arms print (identical dicts)."""
    par = "1 GPU" if ws == 1 else f"{ws} blocks of one {n}x{n}x{n * ws} grid (z split), halos exchanged every step"
    return {"workload": f"Kelvin-Helmholtz {n}^3, FP64, CFL factor 0.05 (reference benchmark problem)",
            "cells_per_gpu": n ** 3, "parallelism": par,
            "l2": "inputs larger than L2 (state ~1 GB per GPU); no flush"}


def timed(solver_like, steps, warm, local):
    """(ms over `steps` steps, clocks) of a Solver / Ensemble after `warm` untimed steps."""
    solver_like.time_steps(max(1, warm))
    with Clocks(local) as ck:
        ms = solver_like.time_steps(steps)
    return ms, ck.summary()


def hbm_roofline(cells, ms_step, hbm_peak, limiter, traffic_per_cell=None):
    ach = B_ALG * cells / (ms_step * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
            "traffic": traffic_per_cell * cells if traffic_per_cell else None, "limiter": limiter}


def e2e_leg(n, precision, K, ws, local):
    """The same metric end to end through mhdgb_step_host: pinned host U in and out every step."""
    import torch
    from mhdturbulence_gb300 import Solver
    with Solver(n, n, n, precision=precision, device=local) as s:
        s.init_kh(seed=1)
        U0 = s.download_cons()
        hin = torch.empty(U0.shape, dtype=torch.float64, pin_memory=True)
        hout = torch.empty(U0.shape, dtype=torch.float64, pin_memory=True)
        hin.numpy()[...] = U0
        a, b = hin.numpy(), hout.numpy()
        s.step_host(a, b, 1)
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(K):
            s.step_host(a, b, 1)
            a, b = b, a
        el = allmax(ws, time.perf_counter() - t0)
    return {"value": replica_value(ws, n ** 3, K, el * 1e3), "unit": "Gcell-updates/s",
            "h2d_bytes_per_step": U0.nbytes, "d2h_bytes_per_step": U0.nbytes,
            "api": "mhdgb_step_host (pinned host U in/out, 1 step per call)", "ms_per_step": el / K * 1e3}


def size_leg(n, K, W, hbm_peak, local):
    """FP64 and mixed KH n^3 on the preferred kernels (no autotuning)."""
    from mhdturbulence_gb300 import Solver
    out = {}
    for prec, k in (("fp64", K), ("mixed", 8 * K)):
        with Solver(n, n, n, precision=prec, device=local) as s:
            s.init_kh(seed=1)
            ms, ck = timed(s, k, W, local)
            r = s.sync()
            cells = n ** 3
            out[prec] = {"value": cells * k / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s", "ms_per_step": ms / k,
                         "ns_per_cell_step": ms / k * 1e6 / cells, "steps": k, "kernel": s.variant_name(),
                         "status": int(r.status), "clocks": ck,
                         "roofline": hbm_roofline(cells, ms / k, hbm_peak,
                                                  "fp64_pipe" if prec == "fp64" else "instruction issue")}
    out["mixed_speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def ensemble_leg(K, W, local, members=64):
    """The batched form: 64 seeded uneven KH grids (per-axis extents from {32, 48, 64, 96, 128}, shear
    Mach U[0.3, 1.5], B_x U[0, 0.3], own noise seeds) in one persistent launch per step, against one
    512^3 KH grid in the mixed form."""
    from mhdturbulence_gb300 import Ensemble, Solver, kh_ensemble_specs
    specs = kh_ensemble_specs(members, seed=2026)
    out = {"members": members, "grids": "per-axis extents from {32,48,64,96,128}, <= 128^3 cells each"}
    for prec, k in (("mixed", 4 * K), ("fp64", max(2, K // 4))):
        with Ensemble(specs, precision=prec, device=local) as ens:
            ens.init_kh()
            ms, ck = timed(ens, k, W, local)
            ens.sync()
            cells = ens.cells
            out["cells"] = cells
            out[prec] = {"value": cells * k / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s", "ms_per_step": ms / k,
                         "steps": k, "kernel": ens.variant_name, "clocks": ck}
    n = 512
    with Solver(n, n, n, precision="mixed", device=local) as s:
        s.init_kh(seed=1)
        k = 2 * K
        ms, ck = timed(s, k, W, local)
        out["single_512_mixed"] = {"value": n ** 3 * k / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s",
                                   "ms_per_step": ms / k, "steps": k, "clocks": ck}
    out["mixed_frac_of_single_512"] = out["mixed"]["value"] / out["single_512_mixed"]["value"]
    return out


def run_decomposed(args, ws, rank, local):
    """N > 1: one KH grid of n x n x (n*N) cells (z in [-N/2, N/2], periodic), one n^3 block per
    rank (mhdturbulence_gb300.distributed), halos of the shared z faces swapped after every step and
    dt / c_h all-reduced: weak scaling with the path's own exchange step.  Halos move over NCCL
    between GPUs (--halo-transport gloo: page-locked host buffers over gloo)."""
    import torch
    import torch.distributed as dist
    from mhdturbulence_gb300.distributed import DistributedGrid, GpuBlock
    dev = local if args.halo_transport == "nccl" else args.device
    torch.cuda.set_device(dev)
    group = dist.new_group(backend="nccl") if args.halo_transport == "nccl" else None
    n, K, W = args.n, args.steps, args.warmup
    nz = n * ws
    domain = ((-0.5, 0.5), (-1.0, 1.0), (-0.5 * ws, 0.5 * ws))
    res = {}
    for prec, k in (("fp64", K), ("mixed", K * args.mixed_factor)):
        blk = GpuBlock(n, n, nz, (1, 1, ws), (0, 0, rank), domain=domain, precision=prec, device=dev,
                       transport="cuda" if args.halo_transport == "nccl" else "cpu")
        blk.init_kh(seed=1)
        g = DistributedGrid(blk, group=group)
        g.prepare()
        g.step(W)
        torch.cuda.synchronize(dev)
        with Clocks(dev) as ck:
            barrier(ws)
            t0 = time.perf_counter()
            g.step(k)
            torch.cuda.synchronize(dev)
            el = allmax(ws, time.perf_counter() - t0)
        r = g.sync()
        res[prec] = {"value": ws * n ** 3 * k / el / 1e9, "ms_per_step": el / k * 1e3, "steps": k,
                     "clocks": ck.summary(), "status": int(r.status), "kernel": blk.solver.variant_name()}
        blk.solver.close()
    e2e = e2e_leg(n, "fp64", max(2, K // 2), ws, dev)
    if rank != 0:
        return
    hbm_peak, peak_kind = peaks()
    fp, mx = res["fp64"], res["mixed"]
    roofline = hbm_roofline(n ** 3, fp["ms_per_step"], hbm_peak, "fp64_pipe")
    roofline["peak_kind"] = peak_kind
    line = {
        "metric": METRIC, "value": fp["value"], "unit": "Gcell-updates/s", "n_gpus": ws, "steps": fp["steps"],
        "warmup": W, "ms_per_step": fp["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded KH initial state, mhdgb_init_kh_block)",
        "kernel": fp["kernel"], "config": bench_config(n, ws), "roofline": roofline,
        "mixed": {"value": mx["value"], "unit": "Gcell-updates/s", "ms_per_step": mx["ms_per_step"],
                  "clocks": mx["clocks"], "kernel": mx["kernel"]},
        "e2e": dict(e2e, api=e2e["api"] + "; each rank's block as an independent grid"),
        "gpu_launches": fp["steps"], "clocks": fp["clocks"], "status": fp["status"], "cpu_baseline": None,
        "halo_transport": args.halo_transport,
    }
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    from mhdturbulence_gb300 import Solver, _lib

    n, K, W = args.n, args.steps, args.warmup
    cells = n ** 3
    hbm_peak, peak_kind = peaks()
    res = {}
    launches = 0
    for prec in ("fp64", "mixed"):
        kk = K if prec == "fp64" else K * args.mixed_factor
        with Solver(n, n, n, precision=prec, device=local) as s:
            s.init_kh(seed=1)
            s.autotune(steps=2)
            name = s.variant_name()
            s.time_steps(W)
            barrier(ws)
            with Clocks(local) as ck:
                ms = s.time_steps(kk)
            r = s.sync()
            barrier(ws)
            ms_max = allmax(ws, ms)
            if prec == "fp64":
                launches = kk
            res[prec] = {"ms": ms_max, "steps": kk, "kernel": name, "clocks": ck.summary(),
                         "status": int(r.status), "device_bytes": s.device_bytes}
            log(f"[bench] {prec}: {ms_max / kk:.3f} ms/step, {name}")

    e2e = e2e_leg(n, "fp64", max(2, K // 2), ws, local)
    e2e_mixed = e2e_leg(n, "mixed", max(4, K), ws, local)

    if rank != 0:
        return
    fp = res["fp64"]
    ms_step = fp["ms"] / fp["steps"]
    value = replica_value(ws, cells, fp["steps"], fp["ms"])
    prof = profile_summary("fused_fp64_150.json")
    traffic = prof.get("dram_bytes_per_cell") if prof else None
    # "bound"/"frac": the HBM roofline of the contract; "limiter": what actually bounds the kernel (the
    # FP64 pipe, whose use is reported under fp64_pipe)
    roofline = hbm_roofline(cells, ms_step, hbm_peak, "fp64_pipe", traffic)
    roofline.update({"peak_kind": peak_kind, "kernel": "k_fused_step<double> (one launch per step)",
                     "bytes_per_cell_alg": B_ALG})
    fp64_rate = None
    rate = ctypes.c_double()
    if _lib.lib().mhdgb_measure_fp64_rate(local, ctypes.byref(rate)) == 0:
        fp64_rate = rate.value
    fp64_pipe = None
    if prof and prof.get("dp_flops_per_cell") and fp64_rate:
        ach = prof["dp_flops_per_cell"] * cells / (ms_step * 1e-3) / 1e9
        fp64_pipe = {"achieved": ach, "peak": fp64_rate, "unit": "GFLOP/s", "frac": ach / fp64_rate,
                     "peak_kind": "measured (DFMA probe, mhdgb_measure_fp64_rate)",
                     "flops_per_cell": prof["dp_flops_per_cell"]}
        if prof.get("fp64_pipe_inst_per_cell"):
            # issue fraction: all FP64-pipe instructions (compares and selects included) against the
            # probe's DFMA issue rate (fp64_rate / 2 instructions per second)
            inst = prof["fp64_pipe_inst_per_cell"] * cells / (ms_step * 1e-3) / 1e9
            fp64_pipe["inst_frac"] = inst / (fp64_rate / 2.0)
            fp64_pipe["pipe_active_ncu"] = prof.get("fp64_pipe_active_ncu")
        # the reference algorithm's own operation count (each add, mul, div, sqrt one flop), counted
        # on the oracle restatement with an instrumented double: the work rate in its terms
        ref_ops = profile_summary("flops_per_cell_oracle.json")
        if ref_ops and ref_ops.get("flops_per_cell"):
            fp64_pipe["reference_flops_per_cell"] = ref_ops["flops_per_cell"]
            fp64_pipe["reference_gflops"] = ref_ops["flops_per_cell"] * cells / (ms_step * 1e-3) / 1e9
    mx = res["mixed"]
    mx_step = mx["ms"] / mx["steps"]
    mx_value = replica_value(ws, cells, mx["steps"], mx["ms"])
    prof_m = profile_summary("fused_mixed_150.json")
    mixed = {"value": mx_value, "unit": "Gcell-updates/s", "ns_per_cell_step": 1.0 / mx_value * ws,
             "ms_per_step": mx_step, "speedup_vs_fp64": mx_value / value, "kernel": mx["kernel"],
             "roofline": hbm_roofline(cells, mx_step, hbm_peak, "instruction issue (see issue)",
                                      prof_m.get("dram_bytes_per_cell") if prof_m else None),
             "clocks": mx["clocks"], "e2e": e2e_mixed}
    if prof_m and prof_m.get("warp_inst_per_cell") and mx["clocks"].get("sm_mhz"):
        # the mixed step's bound is instruction issue: the warp instructions per cell (ncu) against
        # one warp instruction per clock per SM sub-partition (4 per SM) at the sampled SM clock
        import torch
        nsm = torch.cuda.get_device_properties(local).multi_processor_count
        peak = nsm * 4 * mx["clocks"]["sm_mhz"] * 1e6
        ach = prof_m["warp_inst_per_cell"] * (mx_value / ws) * 1e9
        mixed["issue"] = {"achieved": ach / 1e9, "peak": peak / 1e9, "unit": "G warp-instructions/s",
                          "frac": ach / peak, "warp_inst_per_cell": prof_m["warp_inst_per_cell"]}
    if not args.no_error:
        mixed["error_vs_fp64"] = mixed_error(n, args.error_steps, local)
    extra = {}
    if not args.no_extra:
        extra["size_256"] = size_leg(256, max(4, K // 3), W, hbm_peak, local)
        log(f"[bench] 256^3: fp64 {extra['size_256']['fp64']['ms_per_step']:.3f} ms/step, "
            f"mixed {extra['size_256']['mixed']['ms_per_step']:.3f} ms/step")
        extra["ensemble"] = ensemble_leg(K, W, local)
        log(f"[bench] ensemble: mixed {extra['ensemble']['mixed']['value']:.3f} Gcell/s = "
            f"{extra['ensemble']['mixed_frac_of_single_512']:.3f} of one 512^3 grid")
    cpu = None
    if ws == 1 and not args.no_cpu:
        crate, threads, csteps, cel = cpu_oracle_rate(n, args.cpu_seconds)
        cpu = {"value": crate, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
               "sample": f"KH {n}^3 FP64, {csteps} full steps, {cel:.1f} s wall, oracle port (OpenMP)"}
    line = {
        "metric": METRIC, "value": value, "unit": "Gcell-updates/s", "n_gpus": ws, "steps": fp["steps"],
        "warmup": W, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded KH initial state, mhdgb_init_kh)",
        "ns_per_cell_step": ms_step * 1e6 / cells, "kernel": fp["kernel"],
        "config": bench_config(n, ws),
        "roofline": roofline, "fp64_pipe": fp64_pipe, "mixed": mixed, **extra, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": fp["clocks"], "status": fp["status"],
        "published_context": {"value": 1e-9 / PUBLISHED_4XA100_S_PER_CELL_STEP, "unit": "Gcell-updates/s",
                              "what": "4x A100, f90 OpenACC, 150^3 to t=15 (reference README.md:95)"},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    # --grid (cells per axis); --n is the short form for direct runs (torchrun's own parser would
    # take --n as an abbreviation of its options)
    ap.add_argument("--grid", "--n", dest="n", type=int, default=150)
    ap.add_argument("--mixed-factor", type=int, default=8, help="mixed form times steps*factor steps")
    ap.add_argument("--error-steps", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--cpu-seconds-ref", type=float, default=60.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-error", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the 256^3, ensemble and 512^3 legs")
    ap.add_argument("--halo-transport", choices=["nccl", "gloo"], default="nccl",
                    help="N > 1: halos over NCCL between GPUs, or over gloo through host memory")
    ap.add_argument("--device", type=int, default=0, help="N > 1 with gloo halos: the GPU every rank uses")
    ap.add_argument("--only", choices=["fp64", "mixed", "fp64_exact"], help="time one form only (profiling)")
    ap.add_argument("--variant", type=int, default=0, help="tile-shape variant for --only")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ws, rank, local = dist_setup()
    if args.only:
        run_only(args, local)
    elif args.impl == "reference":
        run_reference(args, ws, rank)
    elif ws > 1:
        run_decomposed(args, ws, rank, local)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
