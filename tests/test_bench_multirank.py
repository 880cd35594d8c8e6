"""The multi-rank host logic of bench.py on the CPU (gloo, world size 2): the
max-over-ranks timing that every rank's value is reduced with, and the
reference arm under torchrun, where rank 0 alone runs and prints one JSON
line and every rank exits 0.  The GPU arms are replicas only (no data-path
collective); their device work is covered by the GPU tests."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.barrier_max(1.5 + rank, world)  # rank 1 is the slower one
    finally:
        dist.destroy_process_group()


def test_barrier_max_over_two_ranks():
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        assert dict(out) == {0: 2.5, 1: 2.5}


@pytest.mark.timeout(300)
def test_reference_arm_under_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--elements-per-side", "4", "--steps", "2", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=280)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
