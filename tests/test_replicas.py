"""The multi-GPU path of bench.py is replicas only (independent renders per
rank, no collective on the data path): its host logic on two `gloo` ranks on
the CPU, and the reference arm's ranks other than 0 exiting without work."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench

    # rank r took 100 + 50 r ms for 10 steps of 1,000 samples
    total, value = bench.replica_throughput(100.0 + 50.0 * rank, 1000, 10, world, dist)
    out.put((rank, total, value))
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_every_rank_samples():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, total, value in res:
        assert total == 150.0  # every rank sees the slowest rank's time
        assert abs(value - 1000 * 10 * world / 0.150 / 1e6) < 1e-12



def test_single_process_needs_no_collective():
    sys.path.insert(0, str(ROOT))
    import bench

    total, value = bench.replica_throughput(200.0, 1000, 10, 1)
    assert total == 200.0 and abs(value - 1000 * 10 / 0.2 / 1e6) < 1e-12


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
