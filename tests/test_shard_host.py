"""Particle-range shards on the host, no GPU.

The sharded swarm's contract: a swarm split into shards, each stepping its
own particle range and exchanging one record per iteration (its best
particle's key, cost and vector), moves exactly as the whole swarm.  Checked
here on the oracle (its restatement of a shard: global particle indices for
the random stream, the argmin key, the penalty and the Latin-hypercube
strata), through the package's own loop and exchange:

  - shards in one process, records concatenated, against the whole swarm,
    every iteration, for each sampler, both global-best rules, the
    constrained path and the async run;
  - two gloo ranks (127.0.0.1), each one shard, exchanging through
    ``TorchDistExchange`` (the all-gather the NCCL path runs) inside
    ``sync_loop``: the concatenated state equals the whole swarm's;
  - the exchange's ties: equal costs go to the lowest global index,
    whichever rank holds it;
  - the C ABI's checks of shard arguments, before any device use."""
import ctypes
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from shard_oracle import OracleShard, local_exchange  # noqa: E402

HERE = Path(__file__).resolve().parent
CONS = np.array([[-1, -1, 2, 0, 0], [1, 1, -2, 0, 0], [-1, 0, 0, 0.25, 1]], np.float32)


def _shard_mod():
    sys.path.insert(0, str(HERE.parent / "parallelparticleswarms.jl_gb300"))
    from parallelparticleswarms import shard

    return shard


def test_shard_ranges_cover_the_swarm():
    shard = _shard_mod()
    for n, k in ((1, 1), (10, 3), (1000, 7), (1 << 20, 8), (5, 5)):
        r = shard.shard_ranges(n, k)
        assert len(r) == k and r[0][0] == 0
        assert all(f1 == f0 + c0 for (f0, c0), (f1, _) in zip(r, r[1:]))
        assert sum(c for _, c in r) == n and max(c for _, c in r) - min(c for _, c in r) <= 1
    with pytest.raises(ValueError):
        shard.shard_ranges(3, 4)
    assert shard.record_bytes(100) == 416 and shard.record_bytes(1) == 32 and shard.record_bytes(3) == 32


def _oprob(orc, case):
    obj, D, lo, hi, prm, cons = case
    return orc.OracleProblem(obj, D, np.full(D, lo, np.float32), np.full(D, hi, np.float32), params=prm, cons=cons)


# (objective id, dim, lo, hi, params, constraints), n, shards, sampler, global-best rule
CASES = [
    ((2, 10, -5.12, 5.12, [10.0], None), 3000, 2, 0, 0),
    ((1, 3, -1.0, 10.0, [1.0, 100.0], None), 1000, 3, 0, 1),   # the CPU-backend rule, uneven shards
    ((0, 5, -3.0, 3.0, [], None), 777, 4, 2, 0),                  # Latin hypercube strata over the whole swarm
    ((7, 2, 0.0, 2.0, [2.0, 1.0], CONS), 500, 2, 0, 0),          # the penalty's global particle index
    ((3, 20, -5.0, 5.0, [20.0, 0.2, 1.0], None), 2049, 5, 0, 0),
    ((2, 3, -5.12, 5.12, [10.0], None), 5, 5, 0, 0),              # shards of one particle
]


@pytest.mark.parametrize("case,n,k,sampler,src", CASES,
                         ids=["rastrigin-2shards", "rosenbrock-3shards-pos", "sphere-4shards-lhs",
                              "constrained-2shards", "ackley-5shards", "one-particle-shards"])
def test_oracle_shards_equal_the_whole_swarm(orc, case, n, k, sampler, src):
    shard = _shard_mod()
    oprob = _oprob(orc, case)
    whole = orc.OracleSwarm(oprob, n, 5).init(sampler)
    shards = [OracleShard(orc, oprob, n, f, c, 5, k, gbest_source=src).init(sampler)
              for f, c in shard.shard_ranges(n, k)]
    local_exchange(shards)
    for s in shards:
        s.apply()

    def check(where):
        for key in ("x", "v", "pbest", "pcost", "cost"):
            got = np.concatenate([getattr(s.ref, key) for s in shards], axis=-1)
            assert np.array_equal(got, getattr(whole, key)), f"{where}: {key}"
        for s in shards:
            assert s.ref.gidx == whole.gidx and np.array_equal(s.ref.g, whole.g), where
            assert np.float32(s.ref.gcost) == np.float32(whole.gcost), where

    check("init")
    w = 0.9
    for it in range(25):
        for s in shards:
            s.step(it == 0, w, 0.99, 1.4962, 1.4962)
        local_exchange(shards)
        for s in shards:
            s.apply()
        whole.sync_run(1, w=w, wdamp=0.99, gbest_source=src)
        w = np.float32(np.float32(w) * np.float32(0.99))
        check(f"iteration {it + 1}")


def test_oracle_async_shards_equal_the_whole_swarm(orc):
    shard = _shard_mod()
    n, k = 1500, 3
    oprob = orc.OracleProblem(2, 17, np.full(17, -5.12, np.float32), np.full(17, 5.12, np.float32), params=[10.0])
    lanes = orc.async_lanes(17)[0]
    whole = orc.OracleSwarm(oprob, n, 9).init()
    shards = [OracleShard(orc, oprob, n, f, c, 9, k).init() for f, c in shard.shard_ranges(n, k)]
    local_exchange(shards)
    for s in shards:
        s.apply()
    whole.async_run(40, w=0.7298, wdamp=0.995, lanes=lanes)
    for s in shards:
        s.ref.async_run(40, w=0.7298, wdamp=0.995, lanes=lanes)
        s._publish()
    local_exchange(shards)
    for s in shards:
        s.apply()
    for key in ("x", "v", "pbest", "pcost"):
        assert np.array_equal(np.concatenate([getattr(s.ref, key) for s in shards], axis=-1), getattr(whole, key))
    assert all(s.ref.gidx == whole.gidx and np.array_equal(s.ref.g, whole.g) for s in shards)


# ------------------------------------------------------------------ gloo ranks
def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, n, iters, out):
    sys.path[:0] = [str(HERE), str(HERE.parent / "oracle"), str(HERE.parent / "parallelparticleswarms.jl_gb300")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import pps_oracle as orc
    from parallelparticleswarms import shard
    from shard_oracle import OracleShard

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        D = 12
        oprob = orc.OracleProblem(2, D, np.full(D, -5.12, np.float32), np.full(D, 5.12, np.float32), params=[10.0])
        first, count = shard.shard_ranges(n, world)[rank]
        sh = OracleShard(orc, oprob, n, first, count, 3, world).init()
        ex = shard.TorchDistExchange()
        ex(sh.local, sh.gathered)  # the init's exchange
        sh.apply()
        shard.sync_loop(sh, ex, iters, w=0.8, wdamp=0.995)
        # ties through the same exchange: equal costs, the lower global index wins
        nb = sh.nb
        for owner in (0, 1):
            rec = np.zeros(nb, np.uint8)
            gidx = 10 + rank if owner == 0 else 10 + (1 - rank)  # rank `owner` holds index 10
            rec[0:8] = np.frombuffer(np.uint64(orc.argmin_key(1.25, gidx)).tobytes(), np.uint8)
            rec[8:12] = np.frombuffer(np.float32(1.25).tobytes(), np.uint8)
            rec[16:16 + 4 * D] = np.frombuffer(np.full(D, float(rank), np.float32).tobytes(), np.uint8)
            sh.local.copy_(torch.from_numpy(rec))
            ex(sh.local, sh.gathered)
            probe = orc.OracleSwarm(oprob, 1, 0)
            probe.apply(sh.gathered.numpy())
            out.put(("tie", rank, owner, probe.gidx, float(probe.g[0])))
        out.put(("state", rank, {k: getattr(sh.ref, k).copy() for k in ("x", "v", "pbest", "pcost", "cost")},
                 sh.ref.gidx, sh.ref.g.copy()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_one_swarm(orc):
    world, port, n, iters = 2, _free_port(), 2001, 30
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, n, iters, q)) for r in range(world)]
    for p in procs:
        p.start()
    msgs = [q.get(timeout=180) for _ in range(3 * world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    D = 12
    oprob = orc.OracleProblem(2, D, np.full(D, -5.12, np.float32), np.full(D, 5.12, np.float32), params=[10.0])
    whole = orc.OracleSwarm(oprob, n, 3).init()
    whole.sync_run(iters, w=0.8, wdamp=0.995)
    states = {m[1]: m for m in msgs if m[0] == "state"}
    for key in ("x", "v", "pbest", "pcost", "cost"):
        got = np.concatenate([states[r][2][key] for r in range(world)], axis=-1)
        assert np.array_equal(got, getattr(whole, key)), key
    for r in range(world):
        assert states[r][3] == whole.gidx and np.array_equal(states[r][4], whole.g)
    for m in msgs:
        if m[0] == "tie":
            _, rank, owner, gidx, g0 = m
            assert gidx == 10 and g0 == float(owner), m  # index 10 wins, with its owner's vector


# ------------------------------------------------------------------ C ABI checks
def test_shard_arguments_are_checked_before_device_use(pps):
    from parallelparticleswarms import _lib

    lib = _lib.load()
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(4, np.float32), [10.0], lb=np.full(4, -5.12, np.float32),
                                   ub=np.full(4, 5.12, np.float32))
    pr = prob.to_c()
    h = ctypes.c_void_p()
    for n_global, first, count in ((0, 0, 1), (100, -1, 10), (100, 0, 0), (100, 95, 10), (1 << 33, 0, 10)):
        assert lib.pps_shard_create(ctypes.byref(pr), n_global, first, count, 0, 0, ctypes.byref(h)) == _lib.EINVAL
        assert h.value is None
    lv = pps.ode.lv_problem(np.ones(22, np.float32), nsteps=100, save_every=10)
    plv = lv.to_c()
    assert lib.pps_shard_create(ctypes.byref(plv), 100, 0, 50, 0, 0, ctypes.byref(h)) == _lib.ENOTSUP
    for fn, args in (("pps_shard_step", (1, 0.7, 1.0, 1.4, 1.4)), ("pps_shard_async", (5, 0.7, 1.0, 1.4, 1.4)),
                     ("pps_shard_apply", ()), ("pps_shard_finish", ()), ("pps_shard_record", (None, None, None)),
                     ("pps_shard_bind", (None, None, 1))):
        assert getattr(lib, fn)(None, *args) == _lib.EINVAL, fn
