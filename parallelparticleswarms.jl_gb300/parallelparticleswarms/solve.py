"""init / solve! / solve / reinit! (src/init.jl, src/solve.jl).

Julia's ``solve!`` and ``reinit!`` are spelled ``solve_`` and ``reinit_``.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .algorithms import (BFGS, GPUUniformSampler, GPUUnboundedSampler, HybridPSO, LatinHypercubeSample,
                         ParallelPSOKernel, ParallelSyncPSOKernel, PSOAlgorithm, SimpleLBFGS)
from .problem import OptimizationProblem, evaluate
from .swarm import C1_DEFAULT, C2_DEFAULT, W_DEFAULT, WDAMP_DEFAULT, Swarm


@dataclass
class OptimizationStats:
    time: float = 0.0          # wall seconds of the iteration loop (src/solve.jl:15,26)
    device_ms: float = 0.0     # device time of the loop (CUDA events)
    iterations: int = 0


@dataclass
class OptimizationSolution:
    """SciMLBase.build_solution(...) fields the reference fills (src/solve.jl:54-57)."""

    u: np.ndarray
    objective: float
    original: object = None              # particle positions, (n, dim): a DevicePositions
    stats: OptimizationStats = field(default_factory=OptimizationStats)
    retcode: str = "Default"             # the reference leaves ReturnCode.Default
    alg: object = None


@dataclass
class PSOCache:
    """PSOCache (src/init.jl:1-7): problem, algorithm, device swarm, sampler."""

    prob: OptimizationProblem
    alg: object
    swarm: Swarm
    sampler: object

    @property
    def particles(self) -> dict:
        return self.swarm.state()

    @property
    def gbest(self):
        return self.swarm.gbest()


@dataclass
class HybridPSOCache:
    """HybridPSOCache (src/init.jl:9-13)."""

    pso_cache: PSOCache
    alg: HybridPSO

    @property
    def prob(self):
        return self.pso_cache.prob

    @property
    def swarm(self):
        return self.pso_cache.swarm


def _sampler_code(sampler) -> int:
    if sampler is None:
        return _lib.SAMPLER_AUTO
    if isinstance(sampler, GPUUniformSampler):
        return _lib.SAMPLER_UNIFORM
    if isinstance(sampler, GPUUnboundedSampler):
        return _lib.SAMPLER_UNBOUNDED
    if isinstance(sampler, LatinHypercubeSample):
        return _lib.SAMPLER_LHS
    raise _lib.PPSError(_lib.ENOTSUP, f"sampler {type(sampler).__name__} is not supported on the device")


def _resolve_sampler(prob: OptimizationProblem, sampler):
    # src/init.jl:102-106: infinite bounds always use the unbounded sampler
    lb, ub = prob.lb, prob.ub
    if lb is None or ub is None or (np.all(np.isinf(lb)) and np.all(np.isinf(ub))):
        return GPUUnboundedSampler()
    return sampler if sampler is not None else GPUUniformSampler()


def init(prob: OptimizationProblem, alg, *, sampler=None, seed: int = 0):
    """Allocate the device swarm and sample the initial particles."""
    prob.require_device_objective()
    if isinstance(alg, HybridPSO):
        return HybridPSOCache(init(prob, alg.pso, sampler=sampler, seed=seed), alg)
    if not isinstance(alg, (ParallelSyncPSOKernel, ParallelPSOKernel)):
        raise _lib.ArgumentError(_lib.EINVAL, f"unsupported algorithm {type(alg).__name__}")
    sampler = _resolve_sampler(prob, sampler)
    gpos = isinstance(alg, ParallelSyncPSOKernel) and alg.gbest_from_position
    sw = Swarm(prob, alg.num_particles, seed=seed, gbest_from_position=gpos)
    sw.init(_sampler_code(sampler))
    return PSOCache(prob, alg, sw, sampler)


def reinit_(cache) -> None:
    """reinit!(cache): resample the particles (src/init.jl:117-141)."""
    if isinstance(cache, HybridPSOCache):
        cache = cache.pso_cache
    cache.swarm.init(_sampler_code(cache.sampler))


def _pso_solve(cache: PSOCache, maxiters, w, wdamp, c1, c2) -> OptimizationSolution:
    alg, sw = cache.alg, cache.swarm
    t0 = time.perf_counter()
    if isinstance(alg, ParallelSyncPSOKernel):
        ms = sw.sync_run(maxiters, w, wdamp, c1, c2)
    elif alg.global_update:
        ms = sw.queue_run(maxiters, w, wdamp, c1, c2)
    else:
        ms = sw.async_run(maxiters, w, wdamp, c1, c2)
    t1 = time.perf_counter()
    u, _, _ = sw.gbest()
    obj = float(evaluate(cache.prob, u))  # prob.f(gbest.position, prob.p), src/solve.jl:56
    # sol.original: every particle's position, (n, dim), kept on the device
    # as the reference's get_pos.(particles) is; copied to the host when read
    original = sw.positions_on_device()
    return OptimizationSolution(u=u, objective=obj, original=original,
                                stats=OptimizationStats(time=t1 - t0, device_ms=ms, iterations=int(maxiters)),
                                alg=alg)


def solve_(cache, *, maxiters: int = 100, w: float = W_DEFAULT, wdamp: float = WDAMP_DEFAULT,
           c1: float = C1_DEFAULT, c2: float = C2_DEFAULT, **kwargs) -> OptimizationSolution:
    """solve!(cache; maxiters) (src/solve.jl:5-59, src/hybrid.jl:47-158)."""
    if isinstance(cache, HybridPSOCache):
        from .hybrid import hybrid_solve
        return hybrid_solve(cache, maxiters=maxiters, w=w, wdamp=wdamp, c1=c1, c2=c2, **kwargs)
    if kwargs:
        raise _lib.ArgumentError(_lib.EINVAL, f"unexpected keyword arguments {sorted(kwargs)}")
    return _pso_solve(cache, maxiters, w, wdamp, c1, c2)


def _field(obj, name):
    return obj[name] if isinstance(obj, dict) else getattr(obj, name)


def check_init_bounds(prob: OptimizationProblem):
    """(lb, ub) with missing bounds as -Inf / +Inf (src/utils.jl:310-318)."""
    lb = np.full(prob.dim, -np.inf, np.float32) if prob.lb is None else prob.lb
    ub = np.full(prob.dim, np.inf, np.float32) if prob.ub is None else prob.ub
    return lb, ub


def pso_solve(prob: OptimizationProblem, alg: PSOAlgorithm, *, maxiters: int = 100, **kwargs):
    """pso_solve(prob, alg; maxiters, kwargs...) (src/algorithms.jl:17-28): the algorithm's own loop."""
    return alg.pso_solve(prob, maxiters=maxiters, **kwargs)


def _plugin_solve(prob: OptimizationProblem, alg: PSOAlgorithm, maxiters: int, kwargs) -> OptimizationSolution:
    """solve(prob, ::PSOAlgorithm) (src/solve.jl:69-87): bounds made explicit, the
    algorithm's pso_solve, then u = gbest.position, objective = f(u, p),
    original = every particle's position, stats.time = the reported time."""
    lb, ub = check_init_bounds(prob)
    prob = prob.remake(lb=lb, ub=ub)
    gbest, particles, solve_time = pso_solve(prob, alg, maxiters=maxiters, **kwargs)
    u = np.asarray(_field(gbest, "position"))
    if prob.on_device:
        objective = float(evaluate(prob, u))
    else:
        objective = prob.f(u, prob.p)
    original = [_field(q, "position") for q in particles]
    return OptimizationSolution(u=u, objective=objective, original=original,
                                stats=OptimizationStats(time=float(solve_time), iterations=int(maxiters)), alg=alg)


def solve(prob: OptimizationProblem, alg, *, maxiters: int | None = None, sampler=None, seed: int = 0,
          **kwargs) -> OptimizationSolution:
    """solve(prob, alg; maxiters) = solve!(init(prob, alg)) (src/solve.jl:61-67).

    Any other ``PSOAlgorithm`` runs through its ``pso_solve`` (src/solve.jl:69-87);
    ``sampler`` and ``seed`` reach it as keywords when they are given.
    ``BFGS()`` alone is Broyden's method from u0 (src/bfgs.jl:2-36).
    ``maxiters`` defaults to 100, and to 1000 for ``BFGS()`` as in the reference."""
    if isinstance(alg, BFGS):
        if sampler is not None:
            raise _lib.ArgumentError(_lib.EINVAL, "BFGS() starts from u0: it takes no sampler")
        from .hybrid import bfgs_solve
        return bfgs_solve(prob, alg, maxiters=1000 if maxiters is None else maxiters, **kwargs)
    if maxiters is None:
        maxiters = 100
    if isinstance(alg, PSOAlgorithm) and not isinstance(alg, (ParallelSyncPSOKernel, ParallelPSOKernel, HybridPSO)):
        if sampler is not None:
            kwargs["sampler"] = sampler
        if seed:
            kwargs["seed"] = seed
        return _plugin_solve(prob, alg, maxiters, kwargs)
    cache = init(prob, alg, sampler=sampler, seed=seed)
    try:
        return solve_(cache, maxiters=maxiters, **kwargs)
    finally:
        (cache.pso_cache if isinstance(cache, HybridPSOCache) else cache).swarm.close()


__all__ = ["init", "solve", "solve_", "reinit_", "pso_solve", "check_init_bounds", "PSOCache", "HybridPSOCache",
           "OptimizationSolution", "OptimizationStats", "SimpleLBFGS", "BFGS"]
