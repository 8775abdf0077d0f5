"""The multi-GPU form is replicas only: bench.py launched by torchrun with
N ranks.  Here, on CPU with the gloo backend and world size 2: the reference
arm prints exactly one JSON line (rank 0) and every rank exits 0, and the
barrier / max-over-ranks helpers the GPU arm uses agree across ranks."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--log2n", "16",
           "--steps", "2", "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT,
                       env={**os.environ, "OMP_NUM_THREADS": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0


_WORKER = r'''
import os, sys
sys.path.insert(0, {root!r})
import bench
world, rank, local, pg = bench.dist()
bench.barrier(pg)
v = bench.allmax(pg, 10.0 + rank)
print("RESULT", rank, world, v, flush=True)
pg.destroy_process_group()
'''


def test_barrier_and_max_over_ranks_gloo():
    pytest.importorskip("torch")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = {**os.environ, "WORLD_SIZE": "2", "RANK": str(rank), "LOCAL_RANK": str(rank),
               "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)}
        procs.append(subprocess.Popen([sys.executable, "-c", _WORKER.format(root=str(ROOT))],
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env))
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e[-2000:]
    vals = sorted(float(o.split()[-1]) for o, _ in outs)
    assert vals == [11.0, 11.0]
