"""Multi-process (world size 2, gloo, CPU) tests of bench.py's torchrun path:
replicas only, rank 0 prints the single JSON line, the time reported is the
max over ranks, and no collective touches the data path."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_path):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_setup()
    v = bench.allreduce_max(float(10 + rank), w)
    bench.barrier(w)
    with open("%s.%d" % (out_path, rank), "w") as f:
        json.dump({"world": w, "rank": r, "max": v}, f)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_allreduce_max_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = free_port()
    out = str(tmp_path / "res")
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        d = json.load(open("%s.%d" % (out, r)))
        assert d["world"] == 2 and d["rank"] == r and d["max"] == 11.0


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("torch")
    env = dict(os.environ)
    env["OMP_NUM_THREADS"] = "2"
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--sizes", "64,256"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "FFT/s" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
