"""The benchmark's multi-rank host logic on CPU: two gloo ranks (replicas of
the workload, no data-path collective) agree on the job time as the slowest
rank's, and a single process needs no process group."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank: int, world: int, port: int, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    got = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got))


def test_max_over_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(world))
    assert res == {0: 15.0, 1: 15.0}


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5


def test_rank_shards_are_contiguous_parts_of_one_job():
    """Rank r's rays are shard r of the job's seeded streams: config 0's
    shards are consecutive slices of one shell-ray stream, and config 1's
    secondary rays consecutive slices of one surface-ray stream; shard 0 is
    the single-GPU workload."""
    import numpy as np
    import bench
    from lightsprintsdk_gb300 import scenes
    _, _, a = bench.make_workload("c0", 4096, shard=0)
    _, _, b = bench.make_workload("c0", 4096, shard=1)
    whole = scenes.shell_rays(8192)
    assert np.array_equal(a, whole[:4096]) and np.array_equal(b, whole[4096:])
    v, t, c1a = bench.make_workload("c1", 8192, shard=0)
    _, _, c1b = bench.make_workload("c1", 8192, shard=1)
    sur = scenes.surface_rays(v, t, 8192)
    assert np.array_equal(c1a[4096:], sur[:4096]) and np.array_equal(c1b[4096:], sur[4096:])
    assert not np.array_equal(c1a[:4096], c1b[:4096])   # each rank's own camera image
    _, _, single = bench.make_workload("c1", 8192)
    assert np.array_equal(single, c1a)


def test_gpus_flag_spawns_one_rank_per_gpu(tmp_path):
    """`bench.py --gpus 2` started as one process launches two ranks with
    torch.distributed.run (here the reference arm, which needs no GPU: rank
    0 prints the job's line, rank 1 exits without work) and exits with their
    status."""
    import json
    import subprocess
    import sys
    import bench
    cmd = bench.spawn_command(2, ["--gpus", "2"], 12345)
    assert cmd[1:4] == ["-m", "torch.distributed.run", "--nnodes=1"] and "--nproc-per-node=2" in cmd
    assert "--master-addr=127.0.0.1" in cmd and cmd[-2:] == ["--gpus", "2"]
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--impl", "reference",
                        "--workload", "c0", "--steps", "1", "--warmup", "1"], capture_output=True, text=True,
                       timeout=600, env=env, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1 and lines[0]["impl"] == "reference", r.stdout[-2000:]
