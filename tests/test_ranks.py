"""The N > 1 path of bench.py on CPU ranks (gloo, world size 2).

The multi-GPU design is replicas only: every rank steps its own box and the
ranks meet only for the timing (a barrier on both sides of the timed region
and a max over ranks).  These tests run that host logic with two gloo ranks,
and check that the reference arm leaves the work to rank 0.
"""
import multiprocessing as mp
import os
import socket
import subprocess
import sys

from conftest import REPO


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        assert bench.dist_ready() and bench.world_size() == world
        bench.rank_barrier()
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, "cpu")     # rank 1 is the slow one
        rate = bench.whole_job_rate(1000.0, world, slowest)
        bench.rank_barrier()
        out.put((rank, slowest, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert [g[1] for g in got] == [15.0, 15.0]            # both ranks see the max
    assert all(abs(g[2] - 2 * 1000.0 / 15.0) < 1e-12 for g in got)   # units of all ranks / slowest time


def test_single_process_helpers_are_identities():
    sys.path.insert(0, str(REPO))
    import bench
    assert not bench.dist_ready()
    bench.rank_barrier()
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10.0, 1, 2.0) == 5.0


def test_non_zero_rank_prints_nothing_for_the_reference_arm():
    """Under torchrun only rank 0 runs and prints the reference arm."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "3"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
