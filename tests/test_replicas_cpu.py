"""The N>1 path on the CPU with world_size 2 over gloo: the bench's rank
plumbing (barrier, maximum over ranks of the timed region) in spawned ranks,
and the reference arm launched by torchrun exactly as for N GPUs (rank 0
prints the one JSON line, the other ranks exit 0 without work).  The MPDATA
step itself has no data-path collective: N GPUs run N replicas."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, _ = bench.dist_init(2)
    bench.barrier(ws)
    m = bench.max_over_ranks(10.0 + 5.0 * r, ws)  # rank 1 is the slower one
    with open(os.path.join(out_dir, "r%d.txt" % r), "w") as f:
        f.write("%d %d %.1f" % (ws, r, m))
    torch.distributed.destroy_process_group()


def test_timed_region_is_the_maximum_over_ranks(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        assert (tmp_path / ("r%d.txt" % r)).read_text() == "2 %d 15.0" % r


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3", "--grid", "32", "32", "8", "--ref-slab", "4"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
