"""The multi-GPU path is replicas only: every rank runs an independent solver
and the ranks meet only for a barrier and the max-over-ranks time. Its host
logic is tested here on CPU with gloo, world size 2: the bench's helpers
across two spawned ranks, and the bench's reference arm under
torch.distributed.run (rank 0 alone works and prints one JSON line)."""
import importlib.util
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


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    bench.barrier(world)
    v = bench.allmax(1.5 + rank, world)
    with open(out + str(rank), "w") as f:
        f.write(repr(v))
    dist.destroy_process_group()


def test_allmax_and_barrier_over_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "r")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    assert [float(open(out + str(r)).read()) for r in (0, 1)] == [2.5, 2.5]


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
