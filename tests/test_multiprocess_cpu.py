"""The benchmark's N > 1 path on the host: ranks under torch.distributed with
the gloo backend (the GPU runs use NCCL, one rank per GPU; replicas only, no
collective on the data path). The barrier and the max over ranks of the timed
region, and the reference arm under torchrun: rank 0 alone runs and prints
one line, the other ranks exit 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    m = bench.allreduce_max(w, 1.5 + r)
    bench.barrier(w)
    import torch.distributed as dist
    q.put((r, w, m, dist.get_backend()))
    dist.destroy_process_group()


def test_barrier_and_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    if torch.cuda.is_available():
        pytest.skip("host-only test (a GPU makes the ranks use NCCL)")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 2.5, "gloo"), (1, 2, 2.5, "gloo")]


def test_reference_arm_under_torchrun_prints_one_line():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("host-only test")
    port = _free_port()
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "3"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 1 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
