"""The largest problems each path accepts, against the oracle.

Swarms take 1 <= dim <= 4096 (pps_swarm_create); the synchronous step keeps
the global best and the bounds of every dim in shared memory (48 kB at
4096 dims, more than a block gets without opting in), the async run holds a
particle in at most 32 lanes of 32 dims (dim <= 1024) and refuses more.  At
those limits the state must still match the oracle bit for bit, through
single steps and the graph-replayed run, for the registered kernels, a user
objective and the no-allocation entry point; one past them is refused
before any device work.  Particle indices are 32-bit unsigned (argmin keys,
Philox counters): a swarm of more than 2^31 particles must move its last
particles as the oracle does."""
import ctypes

import numpy as np
import pytest

import user_sources as us
from test_gpu_sync_parity import assert_state_equal

pytestmark = pytest.mark.gpu

MAX_DIM = 4096
ASYNC_MAX_DIM = 1024


def _pair(pps, orc, name, oid, D, n, lo, hi, prm, seed):
    lb, ub = np.full(D, lo, np.float32), np.full(D, hi, np.float32)
    prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm, lb=lb, ub=ub)
    return pps.Swarm(prob, n, seed=seed), orc.OracleSwarm(orc.OracleProblem(oid, D, lb, ub, params=prm), n, seed)


@pytest.mark.parametrize("name,oid,prm,n", [("rastrigin", 2, [10.0], 96), ("rosenbrock", 1, [1.0, 100.0], 33)])
def test_sync_at_max_dim(pps, orc, name, oid, prm, n):
    sw, ref = _pair(pps, orc, name, oid, MAX_DIM, n, -5.12, 5.12, prm, seed=3)
    with sw:
        sw.init()
        ref.init()
        assert_state_equal(sw, ref, "init")
        for it in range(3):
            sw.sync_run(1)
            ref.sync_run(1)
            assert_state_equal(sw, ref, f"iteration {it + 1}")
        sw.sync_run(32)  # one graph-replayed chunk
        ref.sync_run(32)
        assert_state_equal(sw, ref, "graph")


def test_lhs_init_at_max_dim(pps, orc):
    sw, ref = _pair(pps, orc, "sphere", 0, MAX_DIM, 70, -3.0, 3.0, [], seed=5)
    with sw:
        sw.init(pps._lib.SAMPLER_LHS)
        ref.init(orc.SAMPLER_LHS)
        assert_state_equal(sw, ref, "init")
        sw.sync_run(2)
        ref.sync_run(2)
        assert_state_equal(sw, ref, "2 iterations")


def test_async_at_its_max_dim_and_one_past(pps, orc):
    sw, ref = _pair(pps, orc, "rastrigin", 2, ASYNC_MAX_DIM, 50, -5.12, 5.12, [10.0], seed=9)
    with sw:
        sw.init()
        ref.init()
        sw.async_run(6)
        ref.async_run(6)
        assert_state_equal(sw, ref, "async")
    D = ASYNC_MAX_DIM + 1
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(D, np.float32), [10.0], lb=np.full(D, -5.12, np.float32),
                                   ub=np.full(D, 5.12, np.float32))
    with pps.Swarm(prob, 40, seed=1) as sw:
        sw.init()
        with pytest.raises(pps.PPSError, match="1024"):
            sw.async_run(2)


def test_user_objective_at_max_dim(pps, orc):
    D, n = MAX_DIM, 40
    lb, ub = np.full(D, -5.12, np.float32), np.full(D, 5.12, np.float32)
    f = pps.cuda_objective(us.RASTRIGIN)
    prob = pps.OptimizationProblem(f, np.zeros(D, np.float32), [10.0], lb=lb, ub=ub)
    oprob = orc.OracleProblem(0, D, lb, ub, params=[10.0], user=orc.UserObjective(us.RASTRIGIN))
    ref = orc.OracleSwarm(oprob, n, 4)
    with pps.Swarm(prob, n, seed=4) as sw:
        sw.init()
        ref.init(orc.SAMPLER_UNIFORM)
        assert_state_equal(sw, ref, "init")
        sw.sync_run(2)
        ref.sync_run(2)
        assert_state_equal(sw, ref, "2 iterations")
        sw.sync_run(32)
        ref.sync_run(32)
        assert_state_equal(sw, ref, "graph")


def test_noalloc_at_max_dim(pps):
    """pps_sync_run_noalloc at 4096 dims equals pps_sync_run on the same swarm."""
    torch = pytest.importorskip("torch")
    from parallelparticleswarms import _lib

    lib = _lib.load()
    D, n, K, seed = MAX_DIM, 64, 5, 2
    lb, ub = np.full(D, -5.12, np.float32), np.full(D, 5.12, np.float32)
    params = np.array([10.0], np.float32)
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(D, np.float32), params, lb=lb, ub=ub)
    with pps.Swarm(prob, n, seed=seed) as sw:
        sw.init()
        st = sw.state()
        dev = {k: torch.from_numpy(np.ascontiguousarray(np.atleast_2d(st[k]))).cuda()
               for k in ("x", "v", "pbest", "pcost", "cost")}
        dlb, dub = torch.from_numpy(lb).cuda(), torch.from_numpy(ub).cuda()
        g = torch.zeros(D, dtype=torch.float32, device="cuda")
        ds = _lib.DeviceSwarm(n, n, D, dev["x"].data_ptr(), dev["v"].data_ptr(), dev["pbest"].data_ptr(),
                              dev["pcost"].data_ptr(), dev["cost"].data_ptr(), dlb.data_ptr(), dub.data_ptr(),
                              g.data_ptr())
        gcost, gidx = ctypes.c_float(), ctypes.c_int64()
        rc = lib.pps_sync_run_noalloc(2, _lib.fptr(params), 1, ctypes.byref(ds), seed, 0, K, 0.7298, 1.0, 1.4962,
                                      1.4962, 0, None, ctypes.byref(gcost), ctypes.byref(gidx))
        assert rc == 0, lib.pps_last_error()
        sw.sync_run(K)
        want = sw.state()
        for k in ("x", "v", "pbest"):
            assert np.array_equal(dev[k].cpu().numpy(), want[k]), f"{k} differs"
        u, wcost, widx = sw.gbest()
        assert gidx.value == widx and np.float32(gcost.value) == np.float32(wcost)
        assert np.array_equal(g.cpu().numpy(), u)


def test_one_past_max_dim_is_refused(pps):
    D = MAX_DIM + 1
    prob = pps.OptimizationProblem(pps.sphere, np.zeros(D, np.float32), lb=np.full(D, -1.0, np.float32),
                                   ub=np.full(D, 1.0, np.float32))
    with pytest.raises(pps.PPSError, match="4096"):
        pps.Swarm(prob, 8, seed=0)


def test_particle_indices_past_2p31(pps, orc):
    """2^31 + 4113 particles of 1-D Rastrigin (45 GB of state): the first 64
    and the last 4113 particles, whose indices pass the int32 range, match
    oracle shards of those ranges (each given the GPU's global best before
    every step) through init and three iterations, and the global best is the
    lowest-index argmin of all personal bests."""
    n = (1 << 31) + 4113
    D, seed = 1, 21
    lb, ub = np.full(D, -5.12, np.float32), np.full(D, 5.12, np.float32)
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(D, np.float32), [10.0], lb=lb, ub=ub)
    oprob = orc.OracleProblem(2, D, lb, ub, params=[10.0])
    ranges = [(0, 64), (1 << 31, 4113)]
    refs = [orc.OracleSwarm(oprob, count, seed, first=first, nglobal=n) for first, count in ranges]
    fields = (("x", 0), ("v", 1), ("pbest", 2), ("pcost", 3), ("cost", 4))

    def compare(sw, where):
        for name, field in fields:
            full = sw.get(field)
            for (first, count), ref in zip(ranges, refs):
                got = full[..., first:first + count]
                want = getattr(ref, name)
                assert np.array_equal(got, want, equal_nan=True), f"{where}: {name} of particles {first}+ differ"
            del full

    def give_gbest(sw):
        u, c, i = sw.gbest()
        rec = np.zeros((16 + 4 * D + 15) // 16 * 16, np.uint8)
        rec[0:8] = np.frombuffer(np.uint64(orc.argmin_key(np.float32(c), i)).tobytes(), np.uint8)
        rec[8:12] = np.frombuffer(np.float32(c).tobytes(), np.uint8)
        rec[16:16 + 4 * D] = np.frombuffer(np.asarray(u, np.float32).tobytes(), np.uint8)
        for ref in refs:
            ref.apply(rec)

    with pps.Swarm(prob, n, seed=seed) as sw:
        sw.init()
        for ref in refs:
            ref.init()
        compare(sw, "init")
        for it in range(3):
            give_gbest(sw)
            sw.sync_run(1)
            for ref in refs:
                ref.sync_run(1)
            compare(sw, f"iteration {it + 1}")
        pcost = sw.get(3)
        u, c, i = sw.gbest()
        assert i == int(np.argmin(pcost)) and np.float32(c) == pcost.min()
