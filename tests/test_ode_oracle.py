"""The ode_pso restatement on the CPU: RK4 against a float64 integration,
the loss at the truth against the noise level, and a PSO fit recovering the
parameters (parameter_estim_ode!, src/ode_pso.jl:113-170)."""
import numpy as np
import pytest


def oracle_ode_problem(orc, prob):
    """OracleProblem for an ODE-fit pps problem."""
    return orc.ode_fit_problem(prob)


def test_rk4_matches_float64(orc):
    import parallelparticleswarms as pps

    for model, seed in (("lv", 0), ("fhn", 1)):
        prob, truth = pps.ode.synthetic_fit(model, seed)
        op = oracle_ode_problem(orc, prob)
        t32 = op.ode.solve(truth.astype(np.float32))
        p = prob.p
        t64 = pps.ode.trajectory64(model, truth, (p[0], p[1]), p[2], int(p[3]), int(p[4]), p[5])
        assert np.max(np.abs(t32 - t64)) < 1e-4
        nsaves = prob.data.size // 2
        # SSE at the truth ~ 2 * nsaves * sigma^2
        assert op.objective(truth.astype(np.float32)) == pytest.approx(2 * nsaves * 1e-4, rel=0.5)


def test_oracle_ode_pso_recovers_lotka_volterra(orc):
    import parallelparticleswarms as pps

    prob, truth = pps.ode.synthetic_fit("lv", 7)
    op = oracle_ode_problem(orc, prob)
    sw = orc.OracleSwarm(op, 1024, 11).init()
    sw.sync_run(100)
    assert sw.gcost < 1.0
    assert np.allclose(sw.g, truth, rtol=0.1)
