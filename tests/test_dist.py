"""The N > 1 path of bench.py on CPU: N replicas (one per GPU in a real run) each render their own
frames; rank 0 reports rays summed over ranks divided by the slowest rank's time.  Two gloo ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    rays = [3.0e7, 1.0e7][rank]
    ms = [30.0, 50.0][rank]
    q.put((rank, bench.replica_throughput(rays, ms, world, "cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        value, ms = out[r]
        assert ms == pytest.approx(50.0)
        assert value == pytest.approx(4.0e7 / 0.05 / 1e6)


def test_single_rank_needs_no_group():
    import bench
    v, ms = bench.replica_throughput(1e7, 20.0, 1)
    assert v == pytest.approx(500.0) and ms == 20.0


def test_bench_launches_n_replicas():
    """`bench.py --gpus 2` starts two ranks itself (no torchrun), they join one gloo group, and rank 0
    alone prints the aggregate: n_gpus = 2, rays summed over ranks / the slowest rank's time."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--workload", "dist-check"],
                       capture_output=True, text=True, timeout=180, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["n_gpus"] == 2
    assert lines[0]["value"] == pytest.approx(3.0e6 / 0.011 / 1e6)
    assert lines[0]["ms_per_step"] == pytest.approx(11.0)
