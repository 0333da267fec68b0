"""Multi-rank paths on CPU (gloo, world size 2). The traversal shards by rays
with no exchange, so the benchmark runs replicas: its whole-job throughput
is all ranks' rays over the slowest rank's timed total, and the reference
arm runs on rank 0 alone under torchrun."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


_WORKER = """
import json, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
rank, total = int(sys.argv[1]), float(sys.argv[2])
dist.init_process_group("gloo", init_method="tcp://127.0.0.1:{port}", rank=rank, world_size=2)
value, slowest = bench.replica_value(total, 1000, 5, 2, dist, "cpu")
print(json.dumps([value, slowest]))
dist.destroy_process_group()
"""


def test_replica_throughput_uses_the_slowest_rank():
    port = _free_port()
    code = _WORKER.format(root=ROOT, port=port)
    totals = [10.0, 25.0]
    procs = [subprocess.Popen([sys.executable, "-c", code, str(r), str(totals[r])], stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=180)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for value, slowest in outs:
        assert slowest == 25.0
        assert value == pytest.approx(2 * 1000 * 5 / 25e-3 / 1e6)


def test_reference_arm_under_torchrun_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "3", "--rays", "20000", "--tris", "5000"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = []
    for line in r.stdout.splitlines():
        try:
            lines.append(json.loads(line))
        except ValueError:
            pass
    assert len(lines) == 1, r.stdout
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
