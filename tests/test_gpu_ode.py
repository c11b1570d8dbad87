"""ODE-fit swarms (ode_pso) on the GPU vs the oracle."""
import numpy as np
import pytest

from test_gpu_sync_parity import assert_state_equal
from test_ode_oracle import oracle_ode_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model,n,iters", [("lv", 256, 12), ("fhn", 130, 6), ("lv", 1, 3)])
def test_ode_sync_matches_oracle_every_iteration(pps, orc, model, n, iters):
    prob, truth = pps.ode.synthetic_fit(model, 5)
    op = oracle_ode_problem(orc, prob)
    with pps.Swarm(prob, n, seed=9) as sw:
        sw.init()
        ref = orc.OracleSwarm(op, n, 9).init()
        assert_state_equal(sw, ref, "init")
        for it in range(iters):
            sw.sync_run(1)
            ref.sync_run(1)
            assert_state_equal(sw, ref, f"iteration {it + 1}")


@pytest.mark.parametrize("model,n", [("lv", (1 << 18) + 3), ("fhn", (1 << 18) + 70)])
def test_large_ode_swarm_packed_step_matches_oracle(pps, orc, model, n):
    """Swarms of at least 2^18 particles step two particles per thread with
    their RK4 losses packed in f32x2 (kOdePackedMinParticles): the state must
    stay bit-identical to the oracle's scalar arithmetic; n is ragged so the
    last tile's second lane is partly empty."""
    prob, _ = pps.ode.synthetic_fit(model, 11)
    op = oracle_ode_problem(orc, prob)
    with pps.Swarm(prob, n, seed=21) as sw:
        sw.init()
        ref = orc.OracleSwarm(op, n, 21).init()
        assert_state_equal(sw, ref, "init")
        for it in range(2):
            sw.sync_run(1)
            ref.sync_run(1)
            assert_state_equal(sw, ref, f"iteration {it + 1}")


def test_ode_objective_matches_oracle(pps, orc):
    rng = np.random.default_rng(0)
    for model in ("lv", "fhn"):
        prob, truth = pps.ode.synthetic_fit(model, 2)
        op = oracle_ode_problem(orc, prob)
        x = rng.uniform(0, 5, (300, prob.dim)).astype(np.float32)
        x[0] = truth
        got = pps.evaluate(prob, x)
        want = np.array([op.objective(r) for r in x], np.float32)
        assert np.array_equal(got, want, equal_nan=True)


def test_parameter_estim_ode_recovers_truth(pps):
    for model, seed in (("lv", 1), ("fhn", 2)):
        prob, truth = pps.ode.synthetic_fit(model, seed)
        u, cost = pps.ode.parameter_estim_ode(prob, 1024, maxiters=100, seed=seed)
        nsaves = prob.data.size // 2
        assert cost < 10 * 2 * nsaves * 1e-4, (model, cost)
        assert np.allclose(u, truth, rtol=0.15), (model, u, truth)


def test_async_rejects_ode(pps):
    prob, _ = pps.ode.synthetic_fit("lv", 0)
    with pps.Swarm(prob, 64) as sw:
        sw.init()
        with pytest.raises(pps.PPSError):
            sw.async_run(5)
