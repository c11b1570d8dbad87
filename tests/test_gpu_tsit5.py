"""Tsit5 ODE fits on the GPU (the reference's GPUTsit5 at a fixed step,
saves from its continuous extension): bit-exact against the oracle every
iteration on the reference's own LV and FHN benchmark problems, point
evaluation, the 4-parameter FHN fit, parameter recovery, and the routing
(batches refuse Tsit5 fits, the server runs them as swarms of their own)."""
import numpy as np
import pytest

from test_gpu_sync_parity import assert_state_equal
from test_ode_oracle import oracle_ode_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model,n,iters", [("lv", 1000, 10), ("fhn", 333, 8), ("lv", 1, 3)])
def test_tsit5_sync_matches_oracle_every_iteration(pps, orc, model, n, iters):
    prob, _ = pps.ode.reference_benchmark_fit(model)
    op = oracle_ode_problem(orc, prob)
    with pps.Swarm(prob, n, seed=4) as sw:
        sw.init()
        ref = orc.OracleSwarm(op, n, 4).init()
        assert_state_equal(sw, ref, "init")
        for it in range(iters):
            sw.sync_run(1)
            ref.sync_run(1)
            assert_state_equal(sw, ref, f"iteration {it + 1}")
        sw.sync_run(40)  # graph replay
        ref.sync_run(40)
        assert_state_equal(sw, ref, "graph")


def test_tsit5_objective_matches_oracle(pps, orc):
    rng = np.random.default_rng(1)
    for model in ("lv", "fhn"):
        prob, truth = pps.ode.reference_benchmark_fit(model)
        op = oracle_ode_problem(orc, prob)
        x = rng.uniform(0, 5, (500, prob.dim)).astype(np.float32)
        x[0] = truth
        got = pps.evaluate(prob, x)
        want = np.array([op.objective(r) for r in x], np.float32)
        assert np.array_equal(got, want, equal_nan=True)
        assert got[0] < 1e-3


def test_fhn_four_parameter_rk4_fit_matches_oracle(pps, orc):
    """The FHN fit with l as the 4th parameter on the RK4 path, plain and batched."""
    prob, _ = pps.ode.synthetic_fit("fhn", 3)
    prob4 = pps.ode.fhn_problem(prob.data, fit_l=True)
    op = oracle_ode_problem(orc, prob4)
    with pps.Swarm(prob4, 200, seed=2) as sw:
        sw.init()
        ref = orc.OracleSwarm(op, 200, 2).init()
        sw.sync_run(5)
        ref.sync_run(5)
        assert_state_equal(sw, ref, "fhn4 rk4")
        u, c, i = sw.gbest()
    with pps.Batch() as b:
        b.add(prob4, 200, maxiters=5, seed=2)
        b.run()
        bu, bc, bi = b.result(0)
    assert bi == i and np.float32(bc) == np.float32(c) and np.array_equal(bu, u)


def test_tsit5_recovers_reference_benchmark_parameters(pps):
    """The reference's LV benchmark (10,000 particles, 100 iterations, dt = 0.1)."""
    prob, truth = pps.ode.reference_benchmark_fit("lv")
    u, cost = pps.ode.parameter_estim_ode(prob, 10_000, maxiters=100, seed=0)
    assert cost < 0.05
    assert np.allclose(u, truth, rtol=0.05), (u, truth)


def test_tsit5_routing(pps):
    prob, _ = pps.ode.reference_benchmark_fit("lv")
    with pps.Batch() as b:
        with pytest.raises(pps.PPSError):
            b.add(prob, 64, maxiters=5, seed=1)
    with pps.Server(memory_budget=64 << 20, max_launches=2) as srv:
        u, c, i, _ = srv.wait(srv.submit(prob, 256, maxiters=20, seed=5))
    with pps.Swarm(prob, 256, seed=5) as sw:
        sw.init()
        sw.sync_run(20)
        au, ac, ai = sw.gbest()
    assert i == ai and np.float32(c) == np.float32(ac) and np.array_equal(u, au)


# ---------------------------------------------------------------- adaptive steps
@pytest.mark.parametrize("model,n,iters,rtol", [("lv", 1000, 6, 1e-3), ("fhn", 257, 5, 1e-5), ("lv", 33, 4, 1e-6)])
def test_adaptive_tsit5_sync_matches_oracle_every_iteration(pps, orc, model, n, iters, rtol):
    """parameter_estim_ode!(..., Val(true)): adaptive steps per particle (the
    embedded error estimate, the PI controller), bit-exact vs the oracle."""
    prob, _ = pps.ode.reference_benchmark_fit(model)
    prob = pps.ode.adaptive(prob, reltol=rtol, abstol=rtol * 1e-3)
    op = oracle_ode_problem(orc, prob)
    with pps.Swarm(prob, n, seed=6) as sw:
        sw.init()
        ref = orc.OracleSwarm(op, n, 6).init()
        assert_state_equal(sw, ref, "init")
        for it in range(iters):
            sw.sync_run(1)
            ref.sync_run(1)
            assert_state_equal(sw, ref, f"iteration {it + 1}")
        sw.sync_run(33)  # graph replay
        ref.sync_run(33)
        assert_state_equal(sw, ref, "graph")


def test_adaptive_tsit5_objective_matches_oracle(pps, orc):
    """Point evaluation, including parameters that make the solve hard (the
    step-size bound and the no-progress test give +inf on both sides)."""
    rng = np.random.default_rng(3)
    for model in ("lv", "fhn"):
        prob, truth = pps.ode.reference_benchmark_fit(model)
        prob = pps.ode.adaptive(prob, reltol=1e-4, abstol=1e-7)
        op = oracle_ode_problem(orc, prob)
        x = rng.uniform(0, 10 if model == "lv" else 5, (700, prob.dim)).astype(np.float32)
        x[0] = truth
        got = pps.evaluate(prob, x)
        want = np.array([op.objective(r) for r in x], np.float32)
        assert np.array_equal(got, want, equal_nan=True)
        assert got[0] < 1e-4


def test_adaptive_tsit5_recovers_reference_benchmark_parameters(pps):
    prob, truth = pps.ode.reference_benchmark_fit("lv")
    u, cost = pps.ode.parameter_estim_ode(prob, 10_000, maxiters=100, seed=0, adaptive_steps=True)
    assert cost < 0.05
    assert np.allclose(u, truth, rtol=0.05), (u, truth)


def test_adaptive_tsit5_served_equals_alone(pps):
    """The server runs an adaptive fit as a swarm of its own (batches refuse it):
    the same result as the fit solved alone."""
    prob, _ = pps.ode.reference_benchmark_fit("fhn")
    prob = pps.ode.adaptive(prob, reltol=1e-4, abstol=1e-7)
    with pps.Batch() as b:
        with pytest.raises(pps.PPSError):
            b.add(prob, 64, maxiters=5, seed=1)
    with pps.Server(memory_budget=64 << 20, max_launches=2) as srv:
        u, c, i, _ = srv.wait(srv.submit(prob, 300, maxiters=12, seed=8))
    with pps.Swarm(prob, 300, seed=8) as sw:
        sw.init()
        sw.sync_run(12)
        au, ac, ai = sw.gbest()
    assert i == ai and np.float32(c) == np.float32(ac) and np.array_equal(u, au)


@pytest.mark.parametrize("method", ["rk4", "tsit5", "tsit5_adaptive"])
def test_ode_fit_at_the_save_limit_matches_oracle(pps, orc, method):
    """4096 saves (kOdeMaxSaves): the observations (32 KB) and, for Tsit5 at a
    fixed step, the save table behind them (160 KB of dynamic shared memory
    together, above the default 48 KB) -- init, single steps and a graph
    replay bit-identical to the oracle."""
    nsaves = 4096
    t = np.arange(nsaves) * 0.005
    data = pps.ode._dense64("lv", (1.5, 1.0, 3.0, 1.0), (1.0, 1.0), t).astype(np.float32)
    if method == "rk4":
        prob = pps.ode.lv_problem(data, dt=0.005, nsteps=nsaves - 1, save_every=1)
    else:
        prob = pps.ode.lv_problem(data, dt=0.01, nsteps=(nsaves - 1) // 2 + 1, save_every=1, method=method,
                                  save_dt=0.005)
    op = oracle_ode_problem(orc, prob)
    n = 70
    with pps.Swarm(prob, n, seed=6) as sw:
        sw.init()
        ref = orc.OracleSwarm(op, n, 6).init()
        assert_state_equal(sw, ref, "init")
        sw.sync_run(1)
        ref.sync_run(1)
        assert_state_equal(sw, ref, "iteration 1")
        sw.sync_run(3)  # graph replay
        ref.sync_run(3)
        assert_state_equal(sw, ref, "graph")
