"""The N > 1 paths of bench.py on CPU (gloo, world size 2): replicas only, no data-path
collective.  The ranks' reductions (max of the timed region, sum of the work) and the
per-rank GPU selection are checked in spawned gloo processes; the reference arm runs
under torchrun with rank 0 alone printing its line."""
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


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="3,5")
    sys.path.insert(0, ROOT)
    import bench
    r, w, dist = bench.dist_setup()
    try:
        res = (r, w, os.environ["CUDA_VISIBLE_DEVICES"], bench.PHYS_GPU, bench.max_over_ranks(1.0 + r, dist),
               bench.sum_over_ranks(10.0 * (r + 1), dist))
        bench.barrier(dist)
    finally:
        dist.destroy_process_group()
    out.put(res)


def test_rank_reductions_and_device_selection_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][:4] == (0, 2, "3", 3) and res[1][:4] == (1, 2, "5", 5)
    assert all(r[4] == 2.0 and r[5] == 30.0 for r in res)


def test_reference_arm_under_torchrun_world2():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--cpu-iters", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
