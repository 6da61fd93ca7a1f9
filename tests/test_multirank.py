"""The N > 1 path of bench.py on the CPU with the gloo backend: the
max-over-ranks timing, distinct fields per rank, and a whole two-rank run
of the reference arm under torchrun (rank 0 prints the one JSON line)."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _ranks(rank, world, port, out):
    import torch
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(1.0 + rank, world, "cpu")
    f = bench.make_field(8, 2 * rank, "cpu")
    out[rank] = (ms, float(f.sum()))
    torch.distributed.destroy_process_group()


def test_max_over_ranks_and_fields_per_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    with mp.Manager() as m:
        out = m.dict()
        port = free_port()
        ps = [mp.Process(target=_ranks, args=(r, 2, port, out)) for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0       # every rank sees the slowest rank's time
    assert res[0][1] != res[1][1]              # each rank compresses its own field


def test_two_rank_reference_arm_under_torchrun():
    pytest.importorskip("torch")
    from oracle import zoracle
    zoracle.build(ref=False)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--side", "24", "--steps", "2",
           "--warmup", "1", "--T", "2"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=240, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
