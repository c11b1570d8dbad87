"""Parity at the workload sizes themselves, not scaled-down stand-ins.

Every other parity test runs a few thousand particles; these run the sizes
the benchmarks measure, against the oracle, with the same bar (bit-identical
state):

  - synchronous step, 2^20 particles x 100-D Rastrigin and Rosenbrock in
    [-5.12, 5.12]: init and every one of the first iterations (positions,
    velocities, personal bests, costs, global-best index and vector);
  - asynchronous run at 2^20 x 100-D (8 lanes of 14 dims per particle);
  - HybridPSO, 65,536 x 10-D Rosenbrock and Ackley in [-5, 5]: 200 sync
    iterations, then the L-BFGS (from the personal bests) and Broyden (from
    the positions) stages particle by particle (optimum, value, iterations);
  - the batched ODE workload, 512 Lotka-Volterra + 512 FitzHugh-Nagumo fits
    with 256, 1024 or 4096 particles each, 100 iterations: every fit's result
    in the batch equals its solve alone, and a stratified sample of 32 fits
    equals the oracle's solve of that fit.

The oracle runs about 1e7 particle-iterations/s (PSO) and 1e5 (RK4 fits) on
16 host cores, so each case costs seconds."""
import time

import numpy as np
import pytest

from test_gpu_sync_parity import assert_state_equal
from test_ode_oracle import oracle_ode_problem

pytestmark = pytest.mark.gpu

N_LARGE, D_LARGE = 1 << 20, 100


def _box_problem(pps, orc, obj, name, D, lo, hi, prm):
    lb = np.full(D, lo, np.float32)
    ub = np.full(D, hi, np.float32)
    prob = pps.OptimizationProblem(pps.REGISTRY[name], np.zeros(D, np.float32), prm, lb=lb, ub=ub)
    return prob, orc.OracleProblem(obj, D, lb, ub, params=prm)


@pytest.mark.parametrize("obj,name,prm", [(2, "rastrigin", [10.0]), (1, "rosenbrock", [1.0, 100.0])])
def test_sync_2p20_x_100_every_iteration(pps, orc, obj, name, prm):
    prob, oprob = _box_problem(pps, orc, obj, name, D_LARGE, -5.12, 5.12, prm)
    with pps.Swarm(prob, N_LARGE, seed=0) as sw:
        sw.init()
        ref = orc.OracleSwarm(oprob, N_LARGE, 0).init()
        assert_state_equal(sw, ref, "init")
        for it in range(4):
            sw.sync_run(1)
            ref.sync_run(1)
            assert_state_equal(sw, ref, f"iteration {it + 1}")
        # a graph-replayed chunk after the single steps
        sw.sync_run(32)
        ref.sync_run(32)
        assert_state_equal(sw, ref, "iteration 36")


@pytest.mark.parametrize("obj,name,prm", [(2, "rastrigin", [10.0]), (1, "rosenbrock", [1.0, 100.0])])
def test_async_2p20_x_100(pps, orc, obj, name, prm):
    prob, oprob = _box_problem(pps, orc, obj, name, D_LARGE, -5.12, 5.12, prm)
    with pps.Swarm(prob, N_LARGE, seed=1) as sw:
        sw.init()
        ref = orc.OracleSwarm(oprob, N_LARGE, 1).init()
        lanes, slice_ = orc.async_lanes(D_LARGE)
        info = sw.info()
        assert (info.async_lanes, info.async_slice) == (lanes, slice_) == (8, 14)
        sw.async_run(5)
        ref.async_run(5, lanes=lanes)
        assert_state_equal(sw, ref, "async, 5 iterations")


@pytest.mark.parametrize("obj,name,prm", [(1, "rosenbrock", [1.0, 100.0]), (3, "ackley", [20.0, 0.2, 1.0])])
def test_hybrid_65536_x_10(pps, orc, obj, name, prm):
    from parallelparticleswarms import _lib

    n, D = 65536, 10
    prob, oprob = _box_problem(pps, orc, obj, name, D, -5.0, 5.0, prm)
    with pps.Swarm(prob, n, seed=7) as sw:
        sw.init()
        ref = orc.OracleSwarm(oprob, n, 7).init()
        sw.sync_run(200)
        ref.sync_run(200)
        assert_state_equal(sw, ref, "after 200 sync iterations")
        st = sw.state()
        for kind, x0 in (("lbfgs", st["pbest"]), ("bfgs", st["x"])):
            u, f, idx, _ = sw.local_stage(kind, history=10, maxiters=100, armijo_c1=1e-4, gtol=1e-5)
            xo = sw.get(_lib.FIELD_LOCAL_X)
            fo = sw.get(_lib.FIELD_LOCAL_F)
            its = sw.get(_lib.FIELD_LOCAL_ITERS).astype(np.int32)
            rx, rf, rit = orc.lbfgs(oprob, x0, history=10, maxiters=100, armijo_c1=1e-4, gtol=1e-5,
                                    broyden=(kind == "bfgs"))
            bad = np.flatnonzero((fo != rf) | (its != rit) | np.any(xo != rx, axis=0))
            assert bad.size == 0, f"{kind}: {bad.size} particles differ, first {bad[:5]}"
            k = int(np.argmin(rf))
            assert idx == k and np.float32(f) == rf[k] and np.array_equal(u, rx[:, k]), kind


def _ode_workload(pps, count_each=512, seed=0):
    """The batched ODE workload: fit k is synthetic_fit(model, k) with seed k,
    its particle count drawn from {256, 1024, 4096} by a generator seeded 0."""
    rng = np.random.default_rng(seed)
    fits = []
    for k in range(2 * count_each):
        prob, _ = pps.ode.synthetic_fit("lv" if k < count_each else "fhn", k)
        fits.append((prob, int(rng.choice([256, 1024, 4096]))))
    return fits


def test_ode_batch_1024_fits(pps, orc):
    fits = _ode_workload(pps)
    with pps.Batch() as b:
        for k, (p, n) in enumerate(fits):
            b.add(p, n, maxiters=100, seed=k)
        b.run()
        res = [b.result(k) for k in range(len(fits))]
    # every fit alone on the GPU: the same result as in the batch
    differ = []
    for k, (p, n) in enumerate(fits):
        with pps.Swarm(p, n, seed=k) as sw:
            sw.init()
            sw.sync_run(100)
            u, c, i = sw.gbest()
        if not (i == res[k][2] and np.float32(c) == np.float32(res[k][1]) and np.array_equal(u, res[k][0])):
            differ.append(k)
    assert not differ, f"{len(differ)} fits differ batched vs alone, first {differ[:5]}"
    # a stratified sample against the oracle's solve alone
    sample = list(range(0, 512, 32)) + list(range(512, 1024, 32))
    t0 = time.perf_counter()
    for k in sample:
        p, n = fits[k]
        ref = orc.OracleSwarm(oracle_ode_problem(orc, p), n, k).init()
        ref.sync_run(100)
        u, c, i = res[k]
        assert i == ref.gidx and np.float32(c) == np.float32(ref.gcost) and np.array_equal(u, ref.g), \
            f"fit {k} ({p.f.name}, {n} particles) differs from the oracle"
    print(f"oracle: {len(sample)} fits in {time.perf_counter() - t0:.1f} s")
