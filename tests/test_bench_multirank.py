"""bench.py's N>1 launch path on CPU ranks (gloo, world size 2): the barrier and max over ranks of
the timed region, the whole-job value of independent replicas, and the reference arm, which rank 0
alone runs and prints while the other rank exits 0 without work."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, sys
sys.path.insert(0, {root!r})
import bench
ws, rank, local = bench.dist_setup()
bench.barrier(ws)
ms = bench.allmax(ws, 10.0 * (rank + 1))     # rank 1 is the slower one
print(json.dumps({{"rank": rank, "ws": ws, "ms_max": ms, "value": bench.replica_value(ws, 1000, 4, ms)}}))
import torch.distributed as dist
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_and_whole_job_value():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                   LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["ws"] == 2 and o["ms_max"] == 20.0
        assert abs(o["value"] - 2 * 1000 * 4 / 20e-3 / 1e9) < 1e-15


def test_reference_arm_prints_one_line_from_rank_zero():
    port = free_port()
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                        "--impl", "reference", "--gpus", "2", "--grid", "12", "--steps", "2", "--warmup", "3",
                        "--cpu-seconds-ref", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
