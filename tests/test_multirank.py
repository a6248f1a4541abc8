"""The multi-process side of bench.py on CPU (gloo, world size 2): rank
setup, barrier and the max-over-ranks timing reduction, and the reference arm
under torchrun, where rank 0 alone works and prints one line."""
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


def _rank_main(rank, world, port, results):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "CC3D_BENCH_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    results[rank] = bench.max_over_ranks(w, 1.5 + rank)
    bench.barrier(w)
    dist.destroy_process_group()


def test_dist_helpers_gloo_two_ranks():
    import torch.multiprocessing as mp
    mgr = mp.Manager()
    results = mgr.dict()
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, results), nprocs=2, join=True)
    assert dict(results) == {0: 2.5, 1: 2.5}


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_two_ranks():
    env = dict(os.environ, CC3D_BENCH_BACKEND="gloo")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--size", "24",
           "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["cpu_model"]
