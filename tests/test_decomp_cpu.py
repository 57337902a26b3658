"""The block decomposition on CPU ranks: the topology helpers, and world-size 2 and 4 gloo runs of
mhdturbulence_gb300.distributed with oracle-stepped blocks (tests/oracle_block.py) that must equal
the oracle's single-grid run bit for bit: halos paired and ordered correctly (including two
blocks along a periodic axis, which are neighbours across both faces), dt and c_h reduced over all
ranks, uneven splits."""
import json
import os
import socket
import subprocess
import sys

import pytest

from mhdturbulence_gb300 import ic
from mhdturbulence_gb300._lib import BC_EXCHANGE
from mhdturbulence_gb300.domain import block_bc, cart_coords, cart_rank, face_box, neighbour, split_axis

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.join(ROOT, "tests")


def test_cartesian_topology():
    nt = (2, 3, 2)
    for r in range(12):
        assert cart_rank(cart_coords(r, nt), nt) == r
    assert cart_coords(5, nt) == (0, 2, 1)          # row-major, last axis fastest (MPI_Cart_create)
    assert neighbour((0, 0, 1), 0, nt) == (1, 0, 1)  # wraps
    assert neighbour((0, 2, 1), 3, nt) == (0, 0, 1)
    for n, t in ((150, 4), (11, 2), (9, 3), (7, 3)):
        parts = [split_axis(n, t, c) for c in range(t)]
        assert sum(e for _, e in parts) == n
        assert all(parts[c][0] + parts[c][1] == parts[c + 1][0] for c in range(t - 1))
        assert max(e for _, e in parts) - min(e for _, e in parts) <= 1
    # KH: x, z periodic, y reflecting; 2 x 2 x 1 blocks
    assert block_bc(ic.KH_BC, (2, 2, 1), (0, 0, 0)) == (BC_EXCHANGE, BC_EXCHANGE, 2, BC_EXCHANGE, 1, 1)
    assert block_bc(ic.KH_BC, (2, 2, 1), (1, 1, 0)) == (BC_EXCHANGE, BC_EXCHANGE, BC_EXCHANGE, 2, 1, 1)
    ks, js, is_ = face_box((5, 6, 7), 1, ghost=False)
    assert (is_.start, is_.stop, js.start, js.stop, ks.start, ks.stop) == (5, 7, 2, 8, 2, 9)
    ks, js, is_ = face_box((5, 6, 7), 4, ghost=True)
    assert (ks.start, ks.stop, is_.start, is_.stop) == (0, 2, 2, 7)


RANK_SCRIPT = r"""
import json, sys
sys.path[:0] = [{root!r}, {tests!r}, {oracle!r}]
import numpy as np
import torch.distributed as dist
from mhdturbulence_gb300 import ic
from mhdturbulence_gb300.distributed import DistributedGrid
from mhdturbulence_gb300.domain import cart_coords
from oracle_block import OracleBlock
import oracle as O

nx, ny, nz, nt, nsteps, domain, bc = {nx}, {ny}, {nz}, {nt}, {nsteps}, {domain}, {bc}
import datetime
dist.init_process_group("gloo", timeout=datetime.timedelta(seconds=120))
rank = dist.get_rank()
U0 = ic.prim_to_cons(ic.kh_prim(nx, ny, nz, seed=3, domain=domain), 5.0 / 3.0)
blk = OracleBlock(nx, ny, nz, nt, cart_coords(rank, nt), domain=domain, bc=bc)
blk.init_kh_from_whole(U0)
g = DistributedGrid(blk)
g.prepare()
dts = []
for _ in range(nsteps):
    g.step(1)
    r = g.sync()
    dts.append((r.dt, r.chg))
U = g.gather_cons(nx, ny, nz)
if rank == 0:
    orc = O.Oracle(nx, ny, nz, *ic.grid(nx, ny, nz, domain), gam=5.0 / 3.0, bc=bc, spacing_quirk=False)
    Uo, Po = U0.copy(), ic.empty_field(nx, ny, nz, 12)
    orc.update_prim(Uo, Po)
    t, odts, ochgs = orc.run(Uo, Po, nsteps)
    print(json.dumps({{"equal": bool(np.array_equal(U, ic.interior(Uo))),
                      "maxdiff": float(np.abs(U - ic.interior(Uo)).max()),
                      "dts_equal": dts == list(zip(odts.tolist(), ochgs.tolist())),
                      "time_equal": g.sync().time == t}}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_ranks(nt, n=(11, 12, 9), nsteps=6, domain=ic.KH_DOMAIN, bc=ic.KH_BC):
    ws = nt[0] * nt[1] * nt[2]
    port = free_port()
    script = RANK_SCRIPT.format(root=ROOT, tests=TESTS, oracle=os.path.join(ROOT, "oracle"), nx=n[0], ny=n[1],
                                nz=n[2], nt=tuple(nt), nsteps=nsteps, domain=tuple(domain), bc=tuple(bc))
    procs = []
    for rank in range(ws):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                   OMP_NUM_THREADS="1")
        procs.append(subprocess.Popen([sys.executable, "-c", script], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=300)
            assert p.returncode == 0, err[-3000:]
            outs.append(out)
    finally:
        for p in procs:  # a rank that failed must not leave the others waiting
            if p.poll() is None:
                p.kill()
    return json.loads(outs[0].strip().splitlines()[-1])


@pytest.mark.parametrize("nt", [(1, 2, 1), (2, 1, 1), (1, 1, 2)], ids=["y2", "x2-periodic", "z2-periodic"])
def test_two_ranks_equal_single_grid(nt):
    res = run_ranks(nt)
    assert res["equal"], res
    assert res["dts_equal"] and res["time_equal"], res


@pytest.mark.parametrize("nt", [(2, 2, 1), (2, 1, 2)], ids=["x2y2", "x2z2"])
def test_four_ranks_equal_single_grid(nt):
    res = run_ranks(nt)
    assert res["equal"], res
    assert res["dts_equal"] and res["time_equal"], res


def test_four_ranks_mixed_boundaries():
    bc = (ic.BC_OUTFLOW, ic.BC_REFLECTION, ic.BC_PERIODIC, ic.BC_PERIODIC, ic.BC_REFLECTION, ic.BC_OUTFLOW)
    res = run_ranks((1, 2, 2), n=(8, 9, 10), nsteps=5, domain=ic.CUBE_DOMAIN, bc=bc)
    assert res["equal"] and res["dts_equal"] and res["time_equal"], res
