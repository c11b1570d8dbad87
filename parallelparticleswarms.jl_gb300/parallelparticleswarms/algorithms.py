"""Algorithm configuration types (src/algorithms.jl).

``backend`` plays the role of the reference's KernelAbstractions backend
(src/algorithms.jl:78-85,115-121,237-241): the only backend is the GB300
engine ("cuda").  There is no CPU backend and no fallback.
"""
from __future__ import annotations

from dataclasses import dataclass, field

from . import _lib

CUDA = "cuda"


def _check_backend(backend):
    if backend not in (CUDA, None):
        raise _lib.ArgumentError(_lib.EINVAL, f"unsupported backend {backend!r}: this engine runs on CUDA only")
    return CUDA


class PSOAlgorithm:
    """Abstract supertype of the particle-swarm algorithms (src/algorithms.jl:1-15).

    To add an algorithm of one's own, subclass it and implement ``pso_solve``
    (src/algorithms.jl:17-28); ``solve(prob, alg)`` then runs it and builds the
    solution as the reference does for such algorithms (src/solve.jl:69-87).
    The engine's own kernels (``ParallelSyncPSOKernel``, ``ParallelPSOKernel``,
    ``HybridPSO``) do not go through this hook.
    """

    def pso_solve(self, prob, *, maxiters: int, **kwargs):
        """Run the algorithm's loop; return ``(global_best, particles, solve_time)``.

        ``global_best`` exposes ``position`` and ``cost`` (attributes or mapping
        keys), each entry of ``particles`` exposes ``position``, and
        ``solve_time`` is in seconds.
        """
        raise NotImplementedError(f"{type(self).__name__} does not implement pso_solve(prob, *, maxiters, **kwargs)")


@dataclass
class GPUUniformSampler:
    """x = U (ub - lb) + lb (src/utils.jl:57-84)."""


@dataclass
class GPUUnboundedSampler:
    """x = u0 + U |u0|, or U where u0 = 0 (src/utils.jl:23-55)."""


@dataclass
class LatinHypercubeSample:
    """Latin hypercube init (``init(prob, alg; sampler = LatinHypercubeSample())``,
    src/init.jl:15-34): in each dim the n strata of [lb, ub] are dealt to the
    particles by a random permutation, each particle drawing uniformly inside
    its stratum.  Computed on the device (no host sample matrix)."""


@dataclass
class ParallelSyncPSOKernel(PSOAlgorithm):
    """Synchronous PSO: global best recomputed after every iteration
    (src/algorithms.jl:115-121,199-204)."""

    num_particles: int
    backend: str = CUDA
    gbest_from_position: bool = False  # CPU-backend compat, src/lowerlevel_solve.jl:59-60

    def __post_init__(self):
        self.backend = _check_backend(self.backend)
        if int(self.num_particles) < 1:
            raise _lib.ArgumentError(_lib.EINVAL, "num_particles must be >= 1")


@dataclass
class ParallelPSOKernel(PSOAlgorithm):
    """PSO with the update fused into one kernel (src/algorithms.jl:78-85,192-197).
    ``global_update=True`` shares the global best every iteration (the
    reference's queue-lock kernel); ``False`` runs every particle against a
    private best for the whole run in one launch."""

    num_particles: int
    global_update: bool = True
    backend: str = CUDA

    def __post_init__(self):
        self.backend = _check_backend(self.backend)
        if int(self.num_particles) < 1:
            raise _lib.ArgumentError(_lib.EINVAL, "num_particles must be >= 1")


@dataclass
class SimpleLBFGS:
    """Local L-BFGS stage of HybridPSO (projected, backtracking Armijo)."""

    history: int = 10
    armijo_c1: float = 1e-4
    gtol: float = 1e-5
    max_backtracks: int = 30


@dataclass
class BFGS:
    """Local Broyden stage of HybridPSO on grad f = 0 (src/algorithms.jl:216-222)."""

    gtol: float = 1e-5
    max_backtracks: int = 30


class _CpuOnly(PSOAlgorithm):
    """A CPU algorithm of the reference, named so code written for it finds the
    name; this engine has no CPU path, so solving with one raises."""

    def __init__(self, num_particles: int, **kwargs):
        self.num_particles = int(num_particles)

    def pso_solve(self, prob, *, maxiters, **kwargs):
        raise _lib.PPSError(_lib.ENOTSUP, f"{type(self).__name__} is the reference's CPU algorithm and this engine "
                                          "has no CPU path: use ParallelSyncPSOKernel (synchronous) or "
                                          "ParallelPSOKernel (asynchronous / queue-lock) on the GPU")


class ParallelPSOArray(_CpuOnly):
    """The reference's multithreaded CPU swarm over Julia arrays, global best
    updated racily between threads (src/algorithms.jl:123-159,206-208,
    src/lowerlevel_solve.jl:123-181)."""


class SerialPSO(_CpuOnly):
    """The reference's serial CPU swarm, the global best updated particle by
    particle (src/algorithms.jl:161-190,210-212, src/lowerlevel_solve.jl:183-220)."""


@dataclass
class HybridPSO(PSOAlgorithm):
    """Particle-swarm search followed by a local refinement of every particle
    (src/algorithms.jl:225-249, src/hybrid.jl)."""

    pso: PSOAlgorithm = field(default_factory=lambda: ParallelPSOKernel(100, global_update=False))
    local_opt: object = field(default_factory=SimpleLBFGS)
    backend: str = CUDA

    def __post_init__(self):
        self.backend = _check_backend(self.backend)
