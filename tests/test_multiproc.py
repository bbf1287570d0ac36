"""The N > 1 path of bench.py on CPU (gloo, world size 2, 127.0.0.1): the
max-over-ranks timing, the per-rank GPU pinning, and the reference arm under
torch.distributed.run, where rank 0 alone prints the JSON line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="4,5")
    sys.path.insert(0, ROOT)
    import bench
    r, ws, dist = bench.dist_init(2)
    got = bench.barrier_max(dist, 10.0 + 5 * r)
    q.put((r, ws, got, os.environ["CUDA_VISIBLE_DEVICES"]))
    dist.barrier()
    dist.destroy_process_group()


def test_barrier_max_and_gpu_pinning_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[2] for o in out] == [15.0, 15.0]  # every rank sees the max
    assert [o[3] for o in out] == ["4", "5"]    # rank r drives the r-th visible GPU
    assert all(o[1] == 2 for o in out)


def test_reference_arm_under_torchrun_two_ranks():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--fact", "400000", "--dim", "100000", "--cpu-reps", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
