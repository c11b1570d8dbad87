"""Writes oracle_vectors.json: digests of the oracle's outputs on fixed small
cases (sync, CPU-backend global best, async, constraints, the three samplers,
the L-BFGS and Broyden local stages, RK4 and Tsit5 losses, the math functions).
The oracle is pinned against the reference's tests and published vectors
elsewhere; these vectors pin the oracle against itself over time, so a change
that moved the oracle and the kernels together cannot pass unnoticed
(tests/test_oracle_vectors.py recomputes them).  Run from this directory:
``python make_oracle_vectors.py``.

Each digest is the SHA-256 of the little-endian float32 bytes of the named
arrays in order; scalars are stored as their float32 bit patterns.
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
import pps_oracle as orc  # noqa: E402

# the constraint rows of the reference's constraint test (test/constraints.jl), as (c, a, b)
CONS = np.array([[-1, -1, 2, 0, 0], [1, 1, -2, 0, 0], [-1, 0, 0, 0.25, 1]], np.float32)


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(np.asarray(a, np.float32)).astype("<f4").tobytes())
    return h.hexdigest()


def bits(v) -> str:
    return f"{int(np.float32(v).view(np.uint32)):08x}"


def swarm_case(prob, n, seed, iters, sampler=orc.SAMPLER_UNIFORM, mode="sync", gsrc=orc.GBEST_FROM_PBEST):
    sw = orc.OracleSwarm(prob, n, seed).init(sampler)
    if iters:
        if mode == "sync":
            sw.sync_run(iters, w=0.9, wdamp=0.99, gbest_source=gsrc, nthreads=4)
        else:
            sw.async_run(iters, w=0.9, wdamp=0.99, nthreads=4)
    st = sw.state()
    return {"state": digest(st["x"], st["v"], st["pbest"], st["pcost"], st["cost"]), "gcost": bits(sw.gcost),
            "gidx": sw.gidx}


def compute() -> dict:
    orc.load()
    box = lambda D, lo, hi: (np.full(D, lo, np.float32), np.full(D, hi, np.float32))  # noqa: E731
    out = {}
    lb, ub = box(3, -1.0, 10.0)
    rosen3 = orc.OracleProblem(1, 3, lb, ub, params=[1.0, 100.0])
    out["sync_rosenbrock_3d"] = swarm_case(rosen3, 1000, 0, 20)
    out["sync_rosenbrock_3d_gbest_from_position"] = swarm_case(rosen3, 1000, 0, 20, gsrc=orc.GBEST_FROM_POSITION)
    lb, ub = box(100, -5.12, 5.12)
    out["sync_rastrigin_100d"] = swarm_case(orc.OracleProblem(2, 100, lb, ub, params=[10.0]), 256, 7, 20)
    lb, ub = box(20, -5.12, 5.12)
    out["async_rastrigin_20d"] = swarm_case(orc.OracleProblem(2, 20, lb, ub, params=[10.0]), 300, 3, 30, mode="async")
    lb, ub = box(10, -32.0, 32.0)
    out["sync_ackley_10d"] = swarm_case(orc.OracleProblem(3, 10, lb, ub, params=[20.0, 0.2, 1.0]), 500, 5, 15)
    out["sync_constrained_shifted_sphere"] = swarm_case(
        orc.OracleProblem(7, 2, [0, 0], [2, 2], params=[2.0, 1.0], cons=CONS), 1000, 5, 10)
    lb, ub = box(5, -5.12, 5.12)
    out["init_lhs_rastrigin_5d"] = swarm_case(orc.OracleProblem(2, 5, lb, ub, params=[10.0]), 100, 9, 0,
                                              sampler=orc.SAMPLER_LHS)
    u0 = np.array([0.0, 1.5, -2.0, 0.25], np.float32)
    out["init_unbounded_rosenbrock_4d"] = swarm_case(orc.OracleProblem(1, 4, None, None, u0=u0, params=[1.0, 100.0]),
                                                     500, 4, 0, sampler=orc.SAMPLER_UNBOUNDED)

    # local stages from the personal bests (L-BFGS) and positions (Broyden) after 20 iterations
    lb, ub = box(10, -5.0, 5.0)
    rosen10 = orc.OracleProblem(1, 10, lb, ub, params=[1.0, 100.0])
    sw = orc.OracleSwarm(rosen10, 64, 3).init()
    sw.sync_run(20, nthreads=4)
    for name, x0, broyden in (("lbfgs_rosenbrock_10d", sw.pbest, False), ("broyden_rosenbrock_10d", sw.x, True)):
        rx, rf, rit = orc.lbfgs(rosen10, x0, history=10, maxiters=100, gtol=1e-5, broyden=broyden, nthreads=4)
        out[name] = {"x_f": digest(rx, rf), "iters": [int(v) for v in rit]}

    # ODE losses at fixed parameters (RK4 with integer saves; Tsit5 with save_dt)
    t = np.linspace(0, 1, 11, dtype=np.float32)
    data = np.stack([1.0 + 0.5 * np.sin(3 * t), 1.0 + 0.5 * np.cos(2 * t)], axis=1).astype(np.float32)
    for name, model, D, method, fixed in (("lv_rk4", orc.ODE_LV, 4, 0, (0.0,) * 4),
                                         ("lv_tsit5", orc.ODE_LV, 4, 1, (0.0,) * 4),
                                         ("fhn_rk4", orc.ODE_FHN, 3, 0, (0.5, 0.0, 0.0, 0.0)),
                                         ("fhn_tsit5_l", orc.ODE_FHN, 4, 1, (0.0,) * 4)):
        fit = orc.OracleOdeFit(model, D, (1.0, 1.0), 0.01, 100, 10, data, fixed=fixed, method=method, save_dt=0.1)
        p = np.array([1.5, 1.0, 3.0, 1.0][:D], np.float32)
        out[f"ode_loss_{name}"] = {"loss": bits(fit.loss(p)), "trajectory": digest(fit.solve(p))}

    # the math functions on a fixed grid
    L = orc.load()
    xs = np.linspace(-50.0, 50.0, 4001, dtype=np.float32)
    out["cos2pi_sin2pi_exp"] = digest([L.orc_cos2pi(float(x)) for x in xs], [L.orc_sin2pi(float(x)) for x in xs],
                                      [L.orc_exp(float(x) * 0.5) for x in xs])
    return out


if __name__ == "__main__":
    (HERE / "oracle_vectors.json").write_text(json.dumps(compute(), indent=1, sort_keys=True) + "\n")
    print("wrote", HERE / "oracle_vectors.json")
