"""solve!(::HybridPSOCache) (src/hybrid.jl:47-158): the particle swarm, then a
local optimiser on every particle, keeping the local best if it beats the
swarm's."""
from __future__ import annotations

import time

from . import _lib
from .algorithms import BFGS, SimpleLBFGS


def hybrid_solve(cache, *, maxiters=100, w=0.7298, wdamp=1.0, c1=1.4962, c2=1.4962, local_maxiters=50,
                 abstol=None, reltol=None, **kwargs):
    """``abstol`` replaces the local optimiser's gradient-norm tolerance (gtol);
    the local stages have no relative tolerance, so a ``reltol`` is refused
    rather than ignored."""
    from .solve import OptimizationSolution, OptimizationStats, _pso_solve

    if kwargs:
        raise _lib.ArgumentError(_lib.EINVAL, f"unexpected keyword arguments {sorted(kwargs)}")
    if reltol is not None:
        raise _lib.ArgumentError(_lib.EINVAL, "reltol is not supported: the local stages stop on the gradient "
                                              "norm (abstol, else the optimiser's gtol) or after local_maxiters")
    alg = cache.alg
    sol_pso = _pso_solve(cache.pso_cache, maxiters, w, wdamp, c1, c2)
    best_u, best_obj = sol_pso.u, sol_pso.objective
    lo = alg.local_opt
    sw = cache.pso_cache.swarm
    t0 = time.perf_counter()
    if isinstance(lo, SimpleLBFGS):
        gtol = lo.gtol if abstol is None else float(abstol)
        u, f, idx, ms = sw.local_stage("lbfgs", history=lo.history, maxiters=local_maxiters,
                                       armijo_c1=lo.armijo_c1, gtol=gtol, max_backtracks=lo.max_backtracks)
    elif isinstance(lo, BFGS):
        gtol = lo.gtol if abstol is None else float(abstol)
        u, f, idx, ms = sw.local_stage("bfgs", maxiters=local_maxiters, gtol=gtol, max_backtracks=lo.max_backtracks)
    else:
        raise _lib.ArgumentError(_lib.EINVAL, f"unsupported local optimiser {type(lo).__name__}")
    t1 = time.perf_counter()
    if f < best_obj:  # src/hybrid.jl:145-150
        best_u, best_obj = u, f
    return OptimizationSolution(u=best_u, objective=float(best_obj), original=None,
                                stats=OptimizationStats(time=(t1 - t0) + sol_pso.stats.time,
                                                        device_ms=ms + sol_pso.stats.device_ms,
                                                        iterations=int(maxiters)),
                                alg=alg)


def bfgs_solve(prob, alg: BFGS, *, maxiters=1000, abstol=None, reltol=None, **kwargs):
    """solve(prob, BFGS(); maxiters) (src/bfgs.jl:2-36): Broyden's method on
    grad f = 0 from u0 alone, the HybridPSO local stage on a single start
    point.  Like the reference's, it takes no bounds and no constraints: f and
    its gradient are used as they are.  ``abstol`` replaces ``alg.gtol``;
    u = the solver's point, objective = f(u, p) evaluated on the device."""
    from .problem import evaluate
    from .solve import OptimizationSolution, OptimizationStats
    from .swarm import Swarm

    if kwargs:
        raise _lib.ArgumentError(_lib.EINVAL, f"unexpected keyword arguments {sorted(kwargs)}")
    if reltol is not None:
        raise _lib.ArgumentError(_lib.EINVAL, "reltol is not supported: Broyden's method here stops on the "
                                              "gradient norm (abstol, else BFGS.gtol) or after maxiters")
    free = prob.remake(lb=None, ub=None, cons=None)
    gtol = alg.gtol if abstol is None else float(abstol)
    with Swarm(free, 1, seed=0) as sw:
        sw.init()
        sw.set(_lib.FIELD_POSITION, free.u0.reshape(free.dim, 1))
        t0 = time.perf_counter()
        u, _, _, ms = sw.local_stage("bfgs", maxiters=int(maxiters), gtol=gtol, max_backtracks=alg.max_backtracks)
        t1 = time.perf_counter()
    return OptimizationSolution(u=u, objective=float(evaluate(free, u)), original=None,
                                stats=OptimizationStats(time=t1 - t0, device_ms=ms, iterations=int(maxiters)),
                                alg=alg)
