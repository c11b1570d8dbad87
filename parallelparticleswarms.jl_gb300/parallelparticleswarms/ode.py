"""ode_pso: estimate ODE parameters by PSO (src/ode_pso.jl).

An ODE fit is an OptimizationProblem whose objective integrates the model
with the particle's position as its parameters and returns the SSE against
observations (_reduce_losses!, src/ode_pso.jl:47-52).  Two fixed-step
integrators run on the device: the classical RK4 with a save every
``save_every`` steps (the workload's), and Tsitouras' 5(4) pair, the
reference's GPUTsit5 (src/ode_pso.jl:58) with adaptive = false as its
benchmarks run it, saving at t_m = m * save_dt from the method's continuous
extension.  The fit configuration travels in ``p`` = [u0_1, u0_2, dt, nsteps,
save_every, l, method, save_dt] (method 0 = RK4, 1 = Tsit5) and the
observations in ``data`` (nsaves x 2, t = 0 included).

``trajectory64`` / ``synthetic_fit`` build synthetic observations on the host
(float64 RK4 plus Gaussian noise) for the workloads; they are input
generation, not part of the solve.
"""
from __future__ import annotations

import numpy as np

from .problem import OptimizationProblem, fitzhugh_nagumo_fit, lotka_volterra_fit

LV_TRUTH = (1.5, 1.0, 3.0, 1.0)          # benchmarks/Lotka_Volterra/lotka_volterra.jl:16
FHN_TRUTH = (0.7, 0.8, 0.08)             # (a, b, tinv) of benchmarks/Fitzhugh_Nagumo/ode_estimation.jl:14
FHN_L = 0.5                              # l, held fixed


def _rhs64(model: str, p, u, l):
    if model == "lv":
        return np.array([p[0] * u[0] - p[1] * u[0] * u[1], -p[2] * u[1] + p[3] * u[0] * u[1]])
    v, w = u
    return np.array([v - v ** 3 / 3 - w + l, p[2] * (v + p[0] - p[1] * w)])


def trajectory64(model: str, p, u0, dt: float, nsteps: int, save_every: int, l: float = FHN_L) -> np.ndarray:
    """float64 RK4 trajectory at every save_every-th step, t = 0 included."""
    u = np.array(u0, dtype=np.float64)
    p = np.asarray(p, dtype=np.float64)
    out = [u.copy()]
    for s in range(1, nsteps + 1):
        k1 = _rhs64(model, p, u, l)
        k2 = _rhs64(model, p, u + 0.5 * dt * k1, l)
        k3 = _rhs64(model, p, u + 0.5 * dt * k2, l)
        k4 = _rhs64(model, p, u + dt * k3, l)
        u = u + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        if s % save_every == 0:
            out.append(u.copy())
    return np.array(out)


METHODS = {"rk4": 0, "tsit5": 1, "tsit5_adaptive": 2}
RELTOL_DEFAULT, ABSTOL_DEFAULT = 1e-3, 1e-6  # the SciML solvers' default tolerances


def _fit_params(u0, dt, nsteps, save_every, l, method, save_dt, reltol=RELTOL_DEFAULT, abstol=ABSTOL_DEFAULT):
    """The fit configuration vector p.  Adaptive Tsit5 (method 2) integrates to
    (nsaves - 1) save_dt from a first step dt, with reltol / abstol in the
    slots of nsteps / save_every."""
    if method == "tsit5_adaptive":
        if save_dt is None:
            raise ValueError("a Tsit5 fit needs save_dt (the spacing of the observations)")
        return [u0[0], u0[1], dt, float(reltol), float(abstol), l, 2.0, float(save_dt)]
    prm = [u0[0], u0[1], dt, nsteps, save_every, l]
    if method == "tsit5":
        if save_dt is None:
            raise ValueError("a Tsit5 fit needs save_dt (the spacing of the observations)")
        prm += [float(METHODS[method]), float(save_dt)]
    elif method != "rk4":
        raise ValueError(f"method must be one of {sorted(METHODS)}")
    return prm


def lv_problem(data, u0=(1.0, 1.0), dt=0.01, nsteps=1000, save_every=10, lb=0.0, ub=5.0, method="rk4",
               save_dt=None, reltol=RELTOL_DEFAULT, abstol=ABSTOL_DEFAULT) -> OptimizationProblem:
    """Lotka-Volterra fit: du1 = a u1 - b u1 u2, du2 = -c u2 + d u1 u2 (4 parameters)."""
    return OptimizationProblem(lotka_volterra_fit, np.zeros(4, np.float32),
                               _fit_params(u0, dt, nsteps, save_every, 0.0, method, save_dt, reltol, abstol),
                               lb=np.full(4, lb, np.float32), ub=np.full(4, ub, np.float32), data=data)


def fhn_problem(data, u0=(-1.0, 1.0), dt=0.01, nsteps=2000, save_every=10, l=FHN_L, lb=0.0,
                ub=5.0, method="rk4", save_dt=None, fit_l=False, reltol=RELTOL_DEFAULT,
                abstol=ABSTOL_DEFAULT) -> OptimizationProblem:
    """FitzHugh-Nagumo fit of (a, b, tinv), or of (a, b, tinv, l) with ``fit_l``:
    dv = v - v^3/3 - w + l, dw = tinv (v + a - b w)."""
    D = 4 if fit_l else 3
    return OptimizationProblem(fitzhugh_nagumo_fit, np.zeros(D, np.float32),
                               _fit_params(u0, dt, nsteps, save_every, l, method, save_dt, reltol, abstol),
                               lb=np.full(D, lb, np.float32), ub=np.full(D, ub, np.float32), data=data)


def synthetic_fit(model: str, seed: int, noise: float = 0.01, perturb: float = 0.2):
    """One fit of the batched ODE workload: truth = reference parameters times
    U(1 - perturb, 1 + perturb) each, observations = RK4 trajectory + N(0, noise^2).
    LV: u0 = [1, 1], t in [0, 10], 101 points; FHN: u0 = [-1, 1], t in [0, 20], 201 points."""
    rng = np.random.default_rng(seed)
    if model == "lv":
        truth = np.array(LV_TRUTH) * rng.uniform(1 - perturb, 1 + perturb, 4)
        traj = trajectory64("lv", truth, (1.0, 1.0), 0.01, 1000, 10)
        data = (traj + rng.normal(0.0, noise, traj.shape)).astype(np.float32)
        return lv_problem(data), truth
    truth = np.array(FHN_TRUTH) * rng.uniform(1 - perturb, 1 + perturb, 3)
    traj = trajectory64("fhn", truth, (-1.0, 1.0), 0.01, 2000, 10)
    data = (traj + rng.normal(0.0, noise, traj.shape)).astype(np.float32)
    return fhn_problem(data), truth


def _dense64(model: str, p, u0, t_save, h: float = 1e-3, l: float = FHN_L) -> np.ndarray:
    """float64 RK4 at step h, sampled at the times t_save (multiples of h)."""
    p = np.asarray(p, dtype=np.float64)
    u = np.array(u0, dtype=np.float64)
    marks = np.rint(np.asarray(t_save) / h).astype(np.int64)
    out, s = [], 0
    for m in marks:
        while s < m:
            k1 = _rhs64(model, p, u, l)
            k2 = _rhs64(model, p, u + 0.5 * h * k1, l)
            k3 = _rhs64(model, p, u + 0.5 * h * k2, l)
            k4 = _rhs64(model, p, u + h * k3, l)
            u = u + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
            s += 1
        out.append(u.copy())
    return np.array(out)


def reference_benchmark_fit(model: str):
    """The reference's own ode_pso benchmarks (benchmarks/Lotka_Volterra/
    lotka_volterra.jl, benchmarks/Fitzhugh_Nagumo/ode_estimation.jl):
    observations at t = 0:0.01:3 (301 points) from an accurate solve of the
    true model, Tsit5 at dt = 0.1 with saveat = those points (adaptive =
    false), 10,000 particles, 100 iterations.  LV fits (1.5, 1, 3, 1) from
    u0 = [1, 1] on [0, 10]^4; FHN fits (a, b, tinv, l) = (0.7, 0.8, 0.08, 0.5)
    from u0 = [1, 1] on [0, 5]^4.  The observations come from a float64 RK4
    at step 1e-3 (the reference solves with reltol 1e-9 / 1e-6)."""
    t = np.arange(301) * 0.01
    if model == "lv":
        data = _dense64("lv", LV_TRUTH, (1.0, 1.0), t).astype(np.float32)
        return lv_problem(data, u0=(1.0, 1.0), dt=0.1, nsteps=30, save_every=1, lb=0.0, ub=10.0, method="tsit5",
                          save_dt=0.01), np.array(LV_TRUTH)
    truth = (0.7, 0.8, 0.08, 0.5)
    data = _dense64("fhn", truth[:3], (1.0, 1.0), t, l=truth[3]).astype(np.float32)
    return fhn_problem(data, u0=(1.0, 1.0), dt=0.1, nsteps=30, save_every=1, l=0.0, lb=0.0, ub=5.0,
                       method="tsit5", save_dt=0.01, fit_l=True), np.array(truth)


def adaptive(prob: OptimizationProblem, reltol: float = RELTOL_DEFAULT,
             abstol: float = ABSTOL_DEFAULT) -> OptimizationProblem:
    """The same Tsit5 fit with adaptive steps (its dt becomes the first step;
    integrated to (nsaves - 1) save_dt)."""
    p = list(np.asarray(prob.p, np.float64))
    if len(p) < 8 or int(p[6]) not in (METHODS["tsit5"], METHODS["tsit5_adaptive"]):
        raise ValueError("adaptive steps apply to a Tsit5 fit (method='tsit5' with save_dt)")
    p[3], p[4], p[6] = float(reltol), float(abstol), float(METHODS["tsit5_adaptive"])
    return OptimizationProblem(prob.f, prob.u0, p, lb=prob.lb, ub=prob.ub, data=prob.data)


def parameter_estim_ode(prob: OptimizationProblem, n: int, *, maxiters: int = 100, w: float = 0.7298,
                        wdamp: float = 1.0, seed: int = 0, adaptive_steps: bool = False,
                        reltol: float = RELTOL_DEFAULT, abstol: float = ABSTOL_DEFAULT):
    """parameter_estim_ode!(prob, cache, lb, ub, Val(adaptive); maxiters) (src/ode_pso.jl:54-170):
    returns (gbest position, gbest cost).  ``adaptive_steps`` (Val(true),
    :54-111) integrates a Tsit5 fit with adaptive steps at the given tolerances."""
    from .swarm import Swarm

    if adaptive_steps:
        prob = adaptive(prob, reltol, abstol)
    with Swarm(prob, n, seed=seed) as sw:
        sw.init()
        sw.sync_run(maxiters, w=w, wdamp=wdamp)
        u, cost, _ = sw.gbest()
    return u, cost
