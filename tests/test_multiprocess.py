"""The multi-process side of bench.py on CPU ranks (gloo, world size 2).

With --gpus N > 1 the structured workloads run as slabs with ghost-plane
exchanges, SELL as row blocks with an all-gather and the ensemble as one
ensemble per rank (their exchanges are covered by tests/test_slabs.py and
tests/test_sell_shards.py); what every line shares is the barrier around
the timed region and the maximum of the ranks' times, which these tests
run on two gloo ranks.  The reference arm under torchrun prints one line
from rank 0 and lets the other ranks exit without work."""
import json
import os
import socket
import subprocess
import sys


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


WORKER = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import bench
world, rank, local, dist = bench.dist_setup()
assert dist is not None and world == 2
bench.barrier(dist)
t = bench.max_over_ranks(dist, 1.5 + rank)
bench.barrier(dist)
print(json.dumps({{"rank": rank, "world": world, "max": t}}))
dist.destroy_process_group()
"""


def test_barrier_and_max_over_two_gloo_ranks():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err
    lines = [json.loads(o.strip().splitlines()[-1]) for o, _ in outs]
    assert sorted(l["rank"] for l in lines) == [0, 1]
    assert all(l["max"] == 2.5 for l in lines)


def test_reference_arm_under_torchrun_prints_one_line():
    import __graft_entry__
    __graft_entry__.build()
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--workload", "gol_u8_8192", "--steps", "1", "--warmup", "0"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
    assert line["e2e"]["h2d_bytes_per_step"] == 0
