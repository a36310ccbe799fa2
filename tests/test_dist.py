"""The multi-rank path of bench.py on the CPU: gloo process groups of world
size 2 on 127.0.0.1.  bench.py --gpus N runs independent replicas ("replicas
only": the path has no data exchange), so the only collectives are the
barrier and the max over ranks of the timed region."""
import json
import os
import socket
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

torch = pytest.importorskip("torch")


def free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _max_worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world, init_method=f"tcp://127.0.0.1:{port}")
    elapsed = 100.0 + 50.0 * rank  # the slower rank sets the job's time
    m = bench.max_over_ranks(dist, elapsed)
    with open(os.path.join(out, f"r{rank}.json"), "w") as f:
        json.dump({"max": m, "value": bench.replica_throughput(world, 4, m)}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_max_worker, args=(2, free_port(), str(tmp_path)), nprocs=2, join=True)
    r = [json.load(open(tmp_path / f"r{k}.json")) for k in range(2)]
    assert r[0]["max"] == r[1]["max"] == 150.0
    # 2 replicas x 4 solves in the slowest rank's 150 ms
    assert r[0]["value"] == pytest.approx(2 * 4 / 0.150)


def test_max_over_ranks_without_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 12.5) == 12.5


def test_reference_arm_under_torchrun_two_ranks():
    """Rank 0 alone times the CPU reference and prints one JSON line; rank 1
    exits 0 without work.  (--cells-per-side: torchrun takes --n for a
    prefix of its own options.)"""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--cells-per-side", "10", "--ref-warmup-iters", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
