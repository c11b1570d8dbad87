"""Particle-range shards on the GPU: a swarm split into shards, one record
exchange per iteration, moves bit for bit as the whole swarm.

  - shards of one process on this GPU (``LocalShards``, no collective): every
    iteration of the concatenated state, global-best index and vector equals
    the whole swarm's, for even and ragged splits, both samplers that depend
    on the particle index, both global-best rules, the constrained path and
    the async run; also at 2^20 x 100-D;
  - one rank through the NCCL exchange (``ShardedSwarm`` over a one-rank
    process group): the device records go through ncclAllGather;
  - the apply kernel's ties: equal costs go to the lowest global index."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONS = np.array([[-1, -1, 2, 0, 0], [1, 1, -2, 0, 0], [-1, 0, 0, 0.25, 1]], np.float32)


def compare_whole(sh, whole, where):
    """The shards' concatenated state and their global best equal the whole swarm's."""
    got, want = sh.state(), whole.state()
    for k in ("x", "v", "pbest", "pcost", "cost"):
        assert np.array_equal(got[k], want[k], equal_nan=True), f"{where}: {k} differs"
    u, c, i = sh.gbest()
    wu, wc, wi = whole.gbest()
    assert i == wi and np.float32(c) == np.float32(wc) and np.array_equal(u, wu), f"{where}: global best differs"


def _problem(pps, name, D, lo, hi, prm, cons=None):
    return pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm or None,
                                   lb=np.full(D, lo, np.float32), ub=np.full(D, hi, np.float32), cons=cons)


CASES = [
    ("rastrigin", 100, -5.12, 5.12, [10.0], None, 5000, 2, 1, False),
    ("rosenbrock", 3, -1.0, 10.0, [1.0, 100.0], None, 1000, 3, 1, True),     # ragged, CPU-backend rule
    ("sphere", 7, -3.0, 3.0, [], None, 777, 4, 3, False),                    # Latin hypercube
    ("shifted_sphere", 2, 0.0, 2.0, [2.0, 1.0], CONS, 600, 2, 1, False),     # constrained
    ("ackley", 10, -5.0, 5.0, [20.0, 0.2, 1.0], None, 4099, 5, 1, False),
    ("rastrigin", 3, -5.12, 5.12, [10.0], None, 5, 5, 1, False),            # shards of one particle
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-D{c[1]}-n{c[6]}-{c[7]}shards")
def test_local_shards_equal_the_whole_swarm(pps, case):
    name, D, lo, hi, prm, cons, n, k, sampler, gpos = case
    prob = _problem(pps, name, D, lo, hi, prm, cons)
    with pps.Swarm(prob, n, seed=11, gbest_from_position=gpos) as whole, \
            pps.LocalShards(prob, n, k, seed=11, gbest_from_position=gpos) as sh:
        whole.init(sampler)
        sh.init(sampler)
        compare_whole(sh, whole, "init")
        for it in range(12):
            whole.sync_run(1, w=0.9, wdamp=1.0)
            sh.sync_run(1, w=0.9, wdamp=1.0)
            compare_whole(sh, whole, f"iteration {it + 1}")
        # a run of several iterations (damped inertia carried on the device)
        whole.sync_run(40, w=0.8, wdamp=0.99)
        sh.sync_run(40, w=0.8, wdamp=0.99)
        compare_whole(sh, whole, "after 40 more")


def test_local_shards_2p20_x_100(pps):
    """Two shards of the 2^20 x 100-D Rastrigin swarm: init and three
    iterations bit-identical to the whole swarm."""
    prob = _problem(pps, "rastrigin", 100, -5.12, 5.12, [10.0])
    n = 1 << 20
    with pps.Swarm(prob, n, seed=0) as whole, pps.LocalShards(prob, n, 2, seed=0) as sh:
        whole.init()
        sh.init()
        compare_whole(sh, whole, "init")
        for it in range(3):
            whole.sync_run(1)
            sh.sync_run(1)
            compare_whole(sh, whole, f"iteration {it + 1}")


def test_local_shards_async(pps):
    prob = _problem(pps, "rastrigin", 100, -5.12, 5.12, [10.0])
    with pps.Swarm(prob, 3000, seed=2) as whole, pps.LocalShards(prob, 3000, 3, seed=2) as sh:
        whole.init()
        sh.init()
        whole.async_run(30, wdamp=0.995)
        sh.async_run(30, wdamp=0.995)
        compare_whole(sh, whole, "async 30")
        whole.sync_run(5)
        sh.sync_run(5)
        compare_whole(sh, whole, "async 30 + sync 5")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_one_rank_through_nccl(pps):
    """ShardedSwarm's exchange is ncclAllGather of the device records, ordered
    on the shard's stream; with one rank it must leave the swarm exactly as a
    whole swarm."""
    torch = pytest.importorskip("torch")
    import torch.distributed as dist

    os.environ.setdefault("NCCL_NVLS_ENABLE", "0")
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{_free_port()}", rank=0, world_size=1)
    try:
        prob = _problem(pps, "rosenbrock", 20, -5.0, 5.0, [1.0, 100.0])
        with pps.Swarm(prob, 2500, seed=4) as whole, pps.ShardedSwarm(prob, 2500, 0, 1, seed=4) as sh:
            whole.init()
            sh.init()
            compare_whole(sh, whole, "init")
            for rnd in range(3):
                whole.sync_run(10, w=0.75, wdamp=0.99)
                sh.sync_run(10, w=0.75, wdamp=0.99)
                compare_whole(sh, whole, f"round {rnd + 1}")
            torch.cuda.synchronize()
    finally:
        dist.destroy_process_group()


def test_apply_ties_go_to_the_lowest_index(pps):
    """Three records, two with the same lowest cost: the global best is the
    lower global index of those two, with that record's vector."""
    torch = pytest.importorskip("torch")
    from parallelparticleswarms import _lib, shard
    import pps_oracle as orc

    D = 6
    prob = _problem(pps, "sphere", D, -1.0, 1.0, [])
    nb = shard.record_bytes(D)
    recs = np.zeros((3, nb), np.uint8)
    for r, (cost, idx) in enumerate(((0.5, 40), (0.25, 900), (0.25, 77))):
        recs[r, 0:8] = np.frombuffer(np.uint64(orc.argmin_key(cost, idx)).tobytes(), np.uint8)
        recs[r, 8:12] = np.frombuffer(np.float32(cost).tobytes(), np.uint8)
        recs[r, 16:16 + 4 * D] = np.frombuffer(np.full(D, r + 1.0, np.float32).tobytes(), np.uint8)
    gathered = torch.from_numpy(recs.reshape(-1)).cuda()
    with shard.DeviceShard(prob, 1000, 0, 1000, seed=1, gathered=gathered) as sh:
        sh.init()
        sh.apply()
        sh.finish()
        u, c, i = sh.gbest()
    assert i == 77 and np.float32(c) == np.float32(0.25) and np.array_equal(u, np.full(D, 3.0, np.float32))
    # a shard rejects the whole-swarm entry points
    with shard.DeviceShard(prob, 10, 0, 10) as sh:
        sh.init()
        for fn in ("pps_sync_run", "pps_async_run", "pps_queue_run"):
            rc = getattr(sh._lib, fn)(sh._h, 1, 0.7, 1.0, 1.4, 1.4, None)
            assert rc == _lib.ENOTSUP, fn
