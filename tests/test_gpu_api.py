"""The reference-facing API (init / solve! / solve / reinit!) on the GPU:
test/reinit.jl, test/interface.jl-style plumbing, error behaviour and the
device objective evaluation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rosen(pps, D=3, lo=-1.0, hi=10.0):
    return pps.OptimizationProblem(pps.rosenbrock, np.zeros(D, np.float32), [1.0, 100.0],
                                   lb=np.full(D, lo, np.float32), ub=np.full(D, hi, np.float32))


def test_init_reinit_all_cache_kinds(pps):
    """test/reinit.jl:1-50: init + reinit! for every algorithm."""
    prob = rosen(pps)
    for alg in (pps.ParallelPSOKernel(2000), pps.ParallelSyncPSOKernel(2000),
                pps.ParallelPSOKernel(2000, global_update=False)):
        cache = pps.init(prob, alg, seed=123)
        before = cache.swarm.positions().copy()
        sol = pps.solve_(cache, maxiters=10)
        assert sol.u.shape == (3,)
        pps.reinit_(cache)
        assert np.array_equal(cache.swarm.positions(), before)  # same seed -> same sample
        assert cache.swarm.info().iteration == 0
        cache.swarm.close()


def test_solution_fields(pps):
    prob = rosen(pps)
    sol = pps.solve(prob, pps.ParallelSyncPSOKernel(1000), maxiters=100, seed=0)
    assert sol.retcode == "Default"
    assert sol.original.shape == (1000, 3)
    assert np.float32(sol.objective) == np.float32(pps.evaluate(prob, sol.u))
    assert sol.stats.time > 0 and sol.stats.device_ms > 0 and sol.stats.iterations == 100
    lb, ub = prob.lb, prob.ub
    assert np.all(sol.original >= lb) and np.all(sol.original <= ub)


def test_solve_bang_continues(pps, orc):
    """solve!(cache) twice continues the swarm (same as one longer run)."""
    prob = rosen(pps, D=4)
    c1 = pps.init(prob, pps.ParallelSyncPSOKernel(500), seed=2)
    pps.solve_(c1, maxiters=30)
    s1 = pps.solve_(c1, maxiters=30)
    c2 = pps.init(prob, pps.ParallelSyncPSOKernel(500), seed=2)
    s2 = pps.solve_(c2, maxiters=60)
    assert np.array_equal(s1.u, s2.u)
    assert np.array_equal(c1.swarm.positions(), c2.swarm.positions())
    c1.swarm.close()
    c2.swarm.close()


def test_device_objective_matches_oracle(pps, orc):
    rng = np.random.default_rng(3)
    cases = [("sphere", 0, 9, []), ("rosenbrock", 1, 10, [1.0, 100.0]), ("rastrigin", 2, 100, [10.0]),
             ("ackley", 3, 10, [20.0, 0.2, 1.0]), ("beale", 16, 2, []), ("booth", 17, 2, []),
             ("himmelblau", 18, 2, []), ("quadratic", 19, 2, [1000.0]), ("boundary_quadratic", 20, 1, [])]
    for name, oid, D, prm in cases:
        prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm or None)
        oprob = orc.OracleProblem(oid, D, params=prm)
        x = rng.uniform(-5, 5, (257, D)).astype(np.float32)
        got = pps.evaluate(prob, x)
        want = np.array([oprob.objective(row) for row in x], np.float32)
        assert np.array_equal(got, want), name


def test_errors(pps):
    prob = rosen(pps)
    with pytest.raises(pps.ArgumentError):
        pps.solve(prob, pps.ParallelSyncPSOKernel(10), maxiters=-1)
    with pytest.raises(pps.PPSError):
        pps.Swarm(prob, 10).sync_run(5)  # not initialised
    bad = pps.OptimizationProblem(pps.rosenbrock, np.zeros(3, np.float32), lb=np.full(3, 2, np.float32),
                                  ub=np.full(3, 1, np.float32))
    with pytest.raises(pps.ArgumentError):
        pps.solve(bad, pps.ParallelSyncPSOKernel(10))
    with pytest.raises(pps.ArgumentError):
        pps.solve(prob, pps.ParallelSyncPSOKernel(10), maxiters=5, c1=float("nan"))


def test_overflowing_costs_match_oracle(pps, orc):
    """Far outside its usual box Rosenbrock overflows to +inf for almost every
    particle: ties on +inf resolve to the lowest index and the state still
    matches the oracle bit for bit."""
    from test_gpu_sync_parity import assert_state_equal

    D, n = 2, 256
    lb, ub = np.full(D, -1e10, np.float32), np.full(D, 1e10, np.float32)
    prob = pps.OptimizationProblem(pps.rosenbrock, np.zeros(D, np.float32), [1.0, 100.0], lb=lb, ub=ub)
    oprob = orc.OracleProblem(1, D, lb, ub, params=[1.0, 100.0])
    with pps.Swarm(prob, n, seed=1) as sw:
        sw.init()
        ref = orc.OracleSwarm(oprob, n, 1).init()
        assert_state_equal(sw, ref, "init")
        for it in range(5):
            sw.sync_run(1)
            ref.sync_run(1)
            assert_state_equal(sw, ref, f"iteration {it + 1}")


def test_original_is_a_device_snapshot(pps):
    """sol.original stays on the device as a snapshot (the reference's
    get_pos.(particles) is a new device array, src/solve.jl:51-56): it keeps
    the positions of the solve while the swarm runs on or is closed, and reads
    to the host as (n, dim)."""
    D, n = 5, 3000
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(D, np.float32), [10.0],
                                   lb=np.full(D, -5.12, np.float32), ub=np.full(D, 5.12, np.float32))
    cache = pps.init(prob, pps.ParallelSyncPSOKernel(n), seed=3)
    sol = pps.solve_(cache, maxiters=20)
    want = cache.swarm.positions().T.copy()
    assert sol.original.shape == (n, D) and "device" in repr(sol.original)
    pps.solve_(cache, maxiters=30)          # the swarm moves on
    cache.swarm.close()                     # and goes away
    got = np.asarray(sol.original)
    assert got.shape == (n, D) and np.array_equal(got, want)
    assert "host" in repr(sol.original) and np.array_equal(sol.original[7], want[7])


@pytest.mark.parametrize("D,n", [(3, 1000), (100, 777), (1000, 33)])
def test_particle_records_round_trip(pps, D, n):
    """pps_get_particles / pps_set_particles in the reference's SPSOParticle
    layout (src/ParallelParticleSwarms.jl:34-44): the records hold the SoA
    state field by field, and setting them reproduces that state and its
    global best (the argmin of best_cost)."""
    lb, ub = np.full(D, -5.12, np.float32), np.full(D, 5.12, np.float32)
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(D, np.float32), [10.0], lb=lb, ub=ub)
    with pps.Swarm(prob, n, seed=2) as a, pps.Swarm(prob, n, seed=9) as b:
        a.init()
        a.sync_run(10)
        rec = a.particles()
        st = a.state()
        assert np.array_equal(rec["position"], st["x"].T) and np.array_equal(rec["velocity"], st["v"].T)
        assert np.array_equal(rec["best_position"], st["pbest"].T)
        assert np.array_equal(rec["cost"], st["cost"]) and np.array_equal(rec["best_cost"], st["pcost"])
        b.init()
        b.set_particles(rec)
        sb = b.state()
        for k in ("x", "v", "pbest", "pcost", "cost"):
            assert np.array_equal(sb[k], st[k]), k
        ua, ca, ia = a.gbest()
        ub_, cb, ib = b.gbest()
        assert ia == ib and np.float32(ca) == np.float32(cb) and np.array_equal(ua, ub_)


@pytest.mark.parametrize("layout", ["aos", "soa"])
def test_set_particles_on_a_fresh_swarm(pps, layout):
    """Setting the particles of a swarm that was created but never
    initialised: the global best is the argmin of best_cost (lowest index on
    ties), not particle 0 of the zeroed state, and a run continues from it as
    from the same records set after an init."""
    from parallelparticleswarms import _lib

    D, n = 7, 2500
    lb, ub = np.full(D, -5.12, np.float32), np.full(D, 5.12, np.float32)
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(D, np.float32), [10.0], lb=lb, ub=ub)
    with pps.Swarm(prob, n, seed=4) as a, pps.Swarm(prob, n, seed=4) as fresh, pps.Swarm(prob, n, seed=4) as b:
        a.init()
        a.sync_run(6)
        rec = a.particles()
        if layout == "aos":
            fresh.set_particles(rec)
        else:
            soa = np.concatenate([rec["position"].T.ravel(), rec["velocity"].T.ravel(), rec["cost"],
                                  rec["best_position"].T.ravel(), rec["best_cost"]]).astype(np.float32)
            _lib.check(fresh._lib.pps_set_particles(fresh._h, _lib.LAYOUT_SOA, _lib.fptr(soa)))
        u, c, i = fresh.gbest()
        want = int(np.argmin(rec["best_cost"]))
        assert i == want  # the zeroed argmin slot of a fresh swarm would give particle 0
        assert np.float32(c) == rec["best_cost"][want] and np.array_equal(u, rec["best_position"][want])
        b.init()
        b.set_particles(rec)
        fresh.sync_run(5)
        b.sync_run(5)
        sf, sb = fresh.state(), b.state()
        for k in ("x", "v", "pbest", "pcost", "cost"):
            assert np.array_equal(sf[k], sb[k]), k
