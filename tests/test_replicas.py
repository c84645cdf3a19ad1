"""The multi-GPU path of bench.py (independent replicas, one per rank): the
max-over-ranks time and the whole-job throughput, run as two gloo ranks on
the CPU."""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

torch = pytest.importorskip("torch")
import torch.distributed as tdist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, world, rank)
    step_ms = 100.0 + 25.0 * rank                     # rank 1 is the slow replica
    slowest = bench.max_over_ranks(step_ms, "cpu")
    out.put((rank, slowest, bench.replica_throughput(400000, 10, world, slowest)))
    tdist.barrier()
    tdist.destroy_process_group()


def test_two_replicas_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, value in res:
        assert slowest == 125.0
        assert value == pytest.approx(400000 * 10 * 2 / 0.125)


def test_gpus_flag_relaunches_one_rank_per_gpu():
    """bench.py --gpus N outside a distributed launch runs itself under
    torch.distributed.run with N ranks on 127.0.0.1."""
    sys.path.insert(0, ROOT)
    import bench
    cmd = bench.relaunch_command(["--gpus", "4", "--steps", "10"], 4, 29511)
    i = cmd.index("torch.distributed.run")
    assert cmd[i - 1] == "-m"
    assert cmd[cmd.index("--nproc-per-node") + 1] == "4"
    assert cmd[cmd.index("--master-addr") + 1] == "127.0.0.1"
    assert cmd[cmd.index("--master-port") + 1] == "29511"
    assert cmd[-4:] == ["--gpus", "4", "--steps", "10"] and cmd[-5].endswith("bench.py")
