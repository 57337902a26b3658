"""The block-decomposed grid on the GPU.  A decomposed run takes each block's cell faces from the whole
grid and reduces dt / c_h exactly (min and max), so it must equal the single-grid run bit for bit in
every precision: through the in-process domain (one persistent launch per group and step, halos
copied on the device), through the per-handle halo entry points (the multi-process form's building
blocks) in both the fused and the stage path, and through two gloo ranks sharing the GPU."""
import ctypes as C
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
from mhdturbulence_gb300 import Solver, ic
from mhdturbulence_gb300._lib import BC_EXCHANGE
from mhdturbulence_gb300.distributed import block_geometry, sliced_axes
from mhdturbulence_gb300.domain import Domain, block_bc, cart_coords, cart_rank, face_box, neighbour

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GAM = 5.0 / 3.0
N = (36, 28, 20)


def single_run(n, precision, nsteps, U0=None, domain=ic.KH_DOMAIN, bc=ic.KH_BC):
    with Solver(*n, precision=precision, domain=domain, bc=bc) as s:
        if U0 is None:
            s.init_kh(seed=5)
        else:
            s.upload_cons(U0)
        U_init = s.download_cons()
        dts = []
        for _ in range(nsteps):
            s.step(1)
            r = s.sync()
            dts.append((r.dt, r.chg))
        return U_init, ic.interior(s.download_cons()), dts, r.time


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64", "mixed"])
@pytest.mark.parametrize("nt", [(2, 1, 1), (1, 2, 1), (1, 1, 2), (2, 2, 2), (3, 2, 1)],
                         ids=["x2", "y2", "z2", "x2y2z2", "x3y2"])
def test_domain_equals_single_grid(precision, nt):
    nsteps = 21  # a 16-step graph and 5 single launches
    U0, want, dts, t = single_run(N, precision, nsteps)
    with Domain(*N, nt, precision=precision) as d:
        d.upload_cons(U0)
        d.step(nsteps)
        r = d.sync()
        got = ic.interior(d.download_cons())
    assert r.step == nsteps and r.status == 0
    assert np.array_equal(got, want)
    assert (r.dt, r.chg) == dts[-1] and r.time == t


def test_domain_kh_init_and_oracle():
    """The domain's own KH state equals the single grid's, and the separately rounded form equals
    the oracle, every step's dt and c_h included."""
    n, nt, nsteps = (24, 32, 16), (2, 2, 1), 8
    with Domain(*n, nt, precision="fp64_exact") as d:
        d.init_kh(seed=9)
        U0 = d.download_cons()
        got_dts = []
        for _ in range(nsteps):
            d.step(1)
            r = d.sync()
            got_dts.append((r.dt, r.chg))
        got = ic.interior(d.download_cons())
        diag = d.diag()
    with Solver(*n, precision="fp64_exact") as s:
        s.init_kh(seed=9)
        assert np.array_equal(ic.interior(s.download_cons()), ic.interior(U0))
    orc = O.Oracle(*n, *ic.grid(*n), gam=GAM, bc=ic.KH_BC, spacing_quirk=False)
    U, P = U0.copy(), ic.empty_field(*n, 12)
    orc.update_prim(U, P)
    t, dts, chgs = orc.run(U, P, nsteps)
    assert np.array_equal(got, ic.interior(U))
    assert got_dts == list(zip(dts.tolist(), chgs.tolist()))
    assert r.time == t
    assert np.allclose(diag, orc.diag(P), rtol=1e-12, atol=0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_domain_two_groups_on_one_device(precision):
    """Blocks in two groups, each on its own stream (the multi-GPU code path, both groups on
    device 0): the groups' launches, halo copies and reductions are ordered by events."""
    nsteps = 19
    U0, want, dts, t = single_run(N, precision, nsteps)
    with Domain(*N, (2, 2, 1), precision=precision, devices=[0, 0]) as d:
        d.upload_cons(U0)
        d.step(nsteps)
        r = d.sync()
        got = ic.interior(d.download_cons())
        ms = d.time_steps(4)
    assert np.array_equal(got, want)
    assert r.time == t and ms > 0


def test_domain_mixed_boundaries_periodic_cube():
    bc = (ic.BC_OUTFLOW, ic.BC_REFLECTION, ic.BC_PERIODIC, ic.BC_PERIODIC, ic.BC_REFLECTION, ic.BC_OUTFLOW)
    n, nsteps = (20, 22, 18), 12
    U0 = ic.prim_to_cons(ic.random_smooth_prim(*n, seed=4, domain=ic.CUBE_DOMAIN), GAM)
    _, want, dts, t = single_run(n, "fp64", nsteps, U0=U0, domain=ic.CUBE_DOMAIN, bc=bc)
    with Domain(*n, (2, 2, 3), precision="fp64", domain=ic.CUBE_DOMAIN, bc=bc) as d:
        d.upload_cons(U0)
        d.step(nsteps)
        r = d.sync()
        got = ic.interior(d.download_cons())
    assert np.array_equal(got, want) and r.time == t


def _blocks(n, nt, precision, U0):
    blocks = []
    for b in range(nt[0] * nt[1] * nt[2]):
        c = cart_coords(b, nt)
        off, ext = block_geometry(*n, nt, c)
        s = Solver(*ext, precision=precision, bc=block_bc(ic.KH_BC, nt, c))
        s.set_grid(*sliced_axes(*n, ic.KH_DOMAIN, off, ext))
        s.upload_cons(np.array(U0[off[2]:off[2] + ext[2] + 5, off[1]:off[1] + ext[1] + 5, :,
                                  off[0]:off[0] + ext[0] + 5], copy=True))
        s.coords, s.offset, s.extent = c, off, ext
        blocks.append(s)
    return blocks


def _exchange(blocks, nt, dtype):
    bufs = {}
    for q, s in enumerate(blocks):
        for f in range(6):
            if s.cfg.bc[f] == BC_EXCHANGE:
                t = torch.empty(s.halo_bytes(f) // dtype.itemsize, dtype=dtype, device="cuda")
                torch.cuda.synchronize()
                s.halo_pack(f, t.data_ptr())
                bufs[q, f] = t
    for q, s in enumerate(blocks):
        for f in range(6):
            if s.cfg.bc[f] == BC_EXCHANGE:
                src = cart_rank(neighbour(s.coords, f, nt), nt)
                s.halo_unpack(f, bufs[src, f ^ 1].data_ptr())


def _gather(blocks, n):
    out = np.zeros((n[2], n[1], 10, n[0]))
    for s in blocks:
        o, e = s.offset, s.extent
        out[o[2]:o[2] + e[2], o[1]:o[1] + e[1], :, o[0]:o[0] + e[0]] = ic.interior(s.download_cons())
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_halo_entry_points_fused_path(precision):
    """The multi-process form's building blocks driven in one process: pack / unpack of the fused
    step's primitives through device buffers, and the pending reduction replaced by its min / max."""
    nt, nsteps = (2, 2, 1), 9
    U0, want, dts, t = single_run(N, precision, nsteps)
    blocks = _blocks(N, nt, precision, U0)
    dtype = torch.float32 if precision == "mixed" else torch.float64
    try:
        def reduce():
            red = [s.get_reduction() for s in blocks]
            g = (min(a for a, _ in red), max(b for _, b in red))
            for s in blocks:
                s.set_reduction(*g)
        for s in blocks:
            s.prepare()
        _exchange(blocks, nt, dtype)
        reduce()
        for _ in range(nsteps):
            for s in blocks:
                s.step(1)
            _exchange(blocks, nt, dtype)
            reduce()
        r = blocks[0].sync()
        assert np.array_equal(_gather(blocks, N), want)
        assert r.time == t and (r.dt, r.chg) == dts[-1]
    finally:
        for s in blocks:
            s.close()


def test_halo_entry_points_stage_path():
    """The reference-shaped MPI loop on the stage entry points: local ControlTimestep / EvaluateCh
    reduced over blocks and set back, the ghost fill of the non-exchanged faces, then the halos."""
    nt, nsteps = (1, 2, 2), 4
    U0, want, dts, t = single_run(N, "fp64_exact", nsteps)
    blocks = _blocks(N, nt, "fp64_exact", U0)
    try:
        for s in blocks:
            s.UpdatePrimitvP()
        for step in range(nsteps):
            dt = min(s.ControlTimestep() for s in blocks)
            for s in blocks:
                s.set_dt(dt)
                s.SetBoundaryCondition()
            _exchange(blocks, nt, torch.float64)
            chg = max(s.EvaluateCh() for s in blocks)
            assert (dt, chg) == dts[step]
            for s in blocks:
                s.set_chg(chg)
                for dd in (1, 2, 3):
                    s.GetNumericalFluxD(dd)
                s.UpdateConservU()
                s.DampPsi()
                s.UpdatePrimitvP()
        assert np.array_equal(_gather(blocks, N), want)
    finally:
        for s in blocks:
            s.close()


RANK_SCRIPT = r"""
import json, sys
sys.path[:0] = [{root!r}]
import numpy as np
import torch, torch.distributed as dist
from mhdturbulence_gb300 import Solver, ic
from mhdturbulence_gb300.distributed import DistributedGrid, GpuBlock
from mhdturbulence_gb300.domain import cart_coords

n, nt, nsteps, precision = {n}, {nt}, {nsteps}, {precision!r}
import datetime
dist.init_process_group("gloo", timeout=datetime.timedelta(seconds=120))
rank = dist.get_rank()
U0 = np.load({u0!r})
blk = GpuBlock(*n, nt, cart_coords(rank, nt), precision=precision, device=0, transport="cpu")
blk.init_kh_from_whole(U0)
g = DistributedGrid(blk)
g.prepare()
g.step(nsteps)
r = g.sync()
U = g.gather_cons(*n)
if rank == 0:
    np.save({out!r}, U)
    print(json.dumps({{"time": r.time, "dt": r.dt, "chg": r.chg}}))
dist.destroy_process_group()
"""


def test_two_gloo_ranks_share_the_gpu(tmp_path):
    """Two processes, one block each on GPU 0, halos through page-locked host buffers over gloo (the
    kernels of one rank never wait on the other's)."""
    nt, nsteps, precision = (1, 1, 2), 7, "fp64"
    U0, want, dts, t = single_run(N, precision, nsteps)
    u0, out = str(tmp_path / "u0.npy"), str(tmp_path / "out.npy")
    np.save(u0, U0)
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    script = RANK_SCRIPT.format(root=ROOT, n=N, nt=nt, nsteps=nsteps, precision=precision, u0=u0, out=out)
    procs = [subprocess.Popen([sys.executable, "-c", script], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                              env=dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2",
                                       RANK=str(r)))
             for r in range(2)]
    outs = []
    try:
        for p in procs:
            o, e = p.communicate(timeout=300)
            assert p.returncode == 0, e[-3000:]
            outs.append(o)
    finally:
        for p in procs:  # a rank that failed must not leave the other waiting
            if p.poll() is None:
                p.kill()
    res = json.loads(outs[0].strip().splitlines()[-1])
    assert np.array_equal(np.load(out), want)
    assert res["time"] == t and (res["dt"], res["chg"]) == dts[-1]
