"""The multi-GPU bench path on the CPU: two gloo ranks (127.0.0.1), each with
its own swarm seed; the job's time is the slowest rank's and its throughput
counts both ranks' work (weak scaling, no collective on the data path)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "parallelparticleswarms.jl_gb300"))
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from parallelparticleswarms import multi

    r, w, local = multi.rank_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    elapsed_ms = 100.0 + 50.0 * r  # rank 1 is the slow one
    slowest = multi.max_over_ranks(elapsed_ms, dist, "cpu")
    rate = multi.job_throughput(1000.0, w, slowest)
    seeds = [None] * w
    dist.all_gather_object(seeds, multi.swarm_seed(7, r))
    dist.destroy_process_group()
    out.put((r, w, local, slowest, rate, seeds))


def test_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, w, local, slowest, rate, seeds) in enumerate(res):
        assert (rank, w, local) == (r, 2, r)
        assert slowest == 150.0                     # max over ranks
        assert rate == pytest.approx(2000.0 / 0.150)  # both ranks' units over the slowest time
        assert len(set(seeds)) == 2                 # independent swarms


def test_single_process_defaults(monkeypatch):
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "parallelparticleswarms.jl_gb300"))
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from parallelparticleswarms import multi

    assert multi.rank_env() == (0, 1, 0)
    assert multi.max_over_ranks(3.5) == 3.5
    assert multi.swarm_seed(5, 0) == 5
