"""ParallelParticleSwarms on GB300: the reference's solve/init/solve!/reinit!
API over libpps_cuda.so (hand-written sm_103a kernels, C ABI in include/pps.h).

Exports mirror src/ParallelParticleSwarms.jl:102-104.
"""
from ._lib import ArgumentError, PPSError
from .algorithms import (BFGS, CUDA, GPUUniformSampler, GPUUnboundedSampler, HybridPSO, LatinHypercubeSample,
                         ParallelPSOArray, ParallelPSOKernel, ParallelSyncPSOKernel, PSOAlgorithm, SerialPSO,
                         SimpleLBFGS)
from .problem import (REGISTRY, Objective, OptimizationProblem, ackley, beale, booth, boundary_quadratic,
                      cuda_objective, evaluate, fitzhugh_nagumo_fit, himmelblau, lotka_volterra_fit,
                      mlp_regression, quadratic, quadratic_constraint, rastrigin, rosenbrock, shifted_sphere, sphere)
from .solve import (HybridPSOCache, OptimizationSolution, OptimizationStats, PSOCache, init, pso_solve, reinit_,
                    solve, solve_)
from .swarm import Swarm
from .batch import Batch
from .serve import Server
from .shard import LocalShards, ShardedSwarm, shard_ranges
from . import mlp, ode, shard

__all__ = [
    "ParallelPSOKernel", "ParallelSyncPSOKernel", "ParallelPSOArray", "SerialPSO", "PSOAlgorithm", "HybridPSO",
    "SimpleLBFGS", "BFGS",
    "OptimizationProblem", "solve", "solve_", "init", "reinit_", "pso_solve", "GPUUniformSampler",
    "GPUUnboundedSampler",
    "LatinHypercubeSample",
    "PSOCache", "HybridPSOCache", "OptimizationSolution", "OptimizationStats", "Swarm", "PPSError",
    "ArgumentError", "evaluate", "Objective", "REGISTRY", "sphere", "rosenbrock", "rastrigin", "ackley",
    "lotka_volterra_fit", "fitzhugh_nagumo_fit", "mlp_regression", "beale", "booth", "himmelblau",
    "quadratic", "boundary_quadratic", "shifted_sphere", "quadratic_constraint", "cuda_objective", "CUDA",
    "Batch", "Server", "ode", "mlp", "shard", "ShardedSwarm", "LocalShards", "shard_ranges",
]
