"""Tsit5 (the reference's GPUTsit5, Tsitouras 2011) in the ode_pso oracle:
the tableau meets the 17 order-5 conditions, the compiled continuous
extension is the one its own conditions determine, the float32 restatement
follows a float64 Tsit5 and an accurate solution of the reference's
benchmark problems (dt = 0.1, saves every 0.01 from the continuous
extension), and a PSO fit of the reference's LV benchmark recovers the
parameters."""
import numpy as np
import pytest

import tsit5_coefficients as tc
from test_ode_oracle import oracle_ode_problem


def test_tableau_order_conditions():
    res = tc.order5_residuals()
    assert max(abs(v) for v in res.values()) < 1e-13
    assert np.allclose(tc.A.sum(axis=1)[1:], [0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0], atol=1e-15)


def test_compiled_interpolant_is_the_derived_one():
    assert np.abs(tc.derive_interpolant() - tc.LITERALS_R).max() < 1e-9


def _rhs(model, p, u, l):
    if model == "lv":
        return np.array([p[0] * u[0] - p[1] * u[0] * u[1], -p[2] * u[1] + p[3] * u[0] * u[1]])
    return np.array([u[0] - u[0] ** 3 / 3 - u[1] + l, p[2] * (u[0] + p[0] - p[1] * u[1])])


def tsit5_64(model, p, u0, dt, nsteps, save_dt, nsaves, l=0.0):
    """float64 Tsit5 with the derived continuous extension."""
    R = tc.derive_interpolant()
    u = np.array(u0, np.float64)
    out = [u.copy()]
    m = 1
    for n in range(nsteps):
        k = np.zeros((7, 2))
        k[0] = _rhs(model, p, u, l)
        for i in range(1, 7):
            k[i] = _rhs(model, p, u + dt * (tc.A[i, :i] @ k[:i]), l)
        un = u + dt * (tc.B[:6] @ k[:6])
        while m < nsaves and m * save_dt <= (n + 1) * dt + 1e-12:
            th = (m * save_dt - n * dt) / dt
            w = np.array([th * (1 + th * (R[0, 0] + th * (R[0, 1] + th * R[0, 2])))] +
                         [th * th * (R[i, 0] + th * (R[i, 1] + th * R[i, 2])) for i in range(1, 7)])
            out.append(u + dt * (w @ k))
            m += 1
        u = un
    return np.array(out)


@pytest.mark.parametrize("model", ["lv", "fhn"])
def test_oracle_tsit5_follows_float64_and_the_accurate_solution(orc, model):
    import parallelparticleswarms as pps

    prob, truth = pps.ode.reference_benchmark_fit(model)
    op = oracle_ode_problem(orc, prob)
    t32 = op.ode.solve(truth.astype(np.float32))
    p = truth
    t64 = tsit5_64(model, p[:4] if model == "lv" else p[:3], (1.0, 1.0), 0.1, 30, 0.01, 301,
                   l=0.0 if model == "lv" else p[3])
    assert t32.shape == t64.shape == (301, 2)
    assert np.max(np.abs(t32 - t64)) < 2e-5          # float32 rounding only
    # Tsit5 at dt = 0.1 against the accurate observations: 5th-order steps,
    # 4th-order dense output between them
    assert np.max(np.abs(t64 - prob.data.reshape(-1, 2))) < 2e-4
    assert op.objective(truth.astype(np.float32)) < 1e-3


def test_save_points_on_step_ends_match_the_steps(orc):
    """theta = 1 gives b_i(1) = b_i: a save on a step end equals the step's
    value up to the rounding of the interpolant's polynomial."""
    import parallelparticleswarms as pps

    prob, truth = pps.ode.reference_benchmark_fit("lv")
    op = oracle_ode_problem(orc, prob)
    coarse = orc.OracleOdeFit(orc.ODE_LV, 4, (1.0, 1.0), 0.1, 30, 1, prob.data.reshape(-1, 2)[::10], method=1, save_dt=0.1)
    a = op.ode.solve(truth.astype(np.float32))[::10]
    b = coarse.solve(truth.astype(np.float32))
    assert np.max(np.abs(a - b)) < 1e-5


def test_oracle_pso_fits_the_reference_lv_benchmark(orc):
    import parallelparticleswarms as pps

    prob, truth = pps.ode.reference_benchmark_fit("lv")
    op = oracle_ode_problem(orc, prob)
    sw = orc.OracleSwarm(op, 2048, 3).init()
    sw.sync_run(100)
    assert sw.gcost < 0.5
    assert np.allclose(sw.g, truth, rtol=0.15)
