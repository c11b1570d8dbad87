"""The PSOAlgorithm / pso_solve plugin interface (src/algorithms.jl:1-28,
src/solve.jl:69-87): an algorithm that brings its own loop is run by
solve(prob, alg), which builds the solution from what its pso_solve returns.
The first test is the reference's test/interface.jl case; the loop there is
the caller's, so these run without a GPU, except the last, whose objective is
one of the engine's and is evaluated on the device."""
from collections import namedtuple

import numpy as np
import pytest

Best = namedtuple("Best", "position cost")
Particle = namedtuple("Particle", "position")


@pytest.fixture(scope="module")
def mock(pps):
    class MockPSO(pps.PSOAlgorithm):
        """pso_solve returns u0 as the global best and the only particle."""

        def __init__(self):
            self.calls = []

        def pso_solve(self, prob, *, maxiters, **kwargs):
            self.calls.append(dict(prob=prob, maxiters=maxiters, **kwargs))
            position = prob.u0.copy()
            return Best(position, prob.f(position, prob.p)), [Particle(position)], 0.0

    return MockPSO


def test_reference_interface_case(pps, mock):
    # test/interface.jl: OptimizationProblem((u, _) -> sum(abs2, u), [1.0, -2.0], nothing)
    prob = pps.OptimizationProblem(lambda u, _: float(np.sum(np.abs(u) ** 2)), [1.0, -2.0])
    sol = pps.solve(prob, mock())
    assert np.array_equal(sol.u, prob.u0)
    assert sol.objective == 5.0
    assert len(sol.original) == 1 and np.array_equal(sol.original[0], prob.u0)
    assert sol.stats.time == 0.0
    assert sol.retcode == "Default"


def test_bounds_are_made_explicit_and_keywords_pass_through(pps, mock):
    # check_init_bounds (src/utils.jl:310-318): missing bounds reach pso_solve as -Inf / +Inf
    alg = mock()
    prob = pps.OptimizationProblem(lambda u, p: float(u @ u) * p[0], [0.5, 0.5, 0.5], p=[2.0])
    sol = pps.solve(prob, alg, maxiters=7, seed=3, sampler=pps.LatinHypercubeSample(), extra="x")
    call = alg.calls[-1]
    assert call["maxiters"] == 7 and call["seed"] == 3 and call["extra"] == "x"
    assert isinstance(call["sampler"], pps.LatinHypercubeSample)
    assert np.all(np.isneginf(call["prob"].lb)) and np.all(np.isposinf(call["prob"].ub))
    assert sol.objective == pytest.approx(1.5)
    # given bounds are kept
    bounded = pps.OptimizationProblem(lambda u, p: 0.0, [0.0, 0.0], lb=[-1, -2], ub=[3, 4])
    pps.solve(bounded, alg)
    assert np.array_equal(alg.calls[-1]["prob"].lb, [-1, -2]) and np.array_equal(alg.calls[-1]["prob"].ub, [3, 4])
    assert alg.calls[-1]["maxiters"] == 100 and "seed" not in alg.calls[-1]


def test_mapping_results_and_module_level_pso_solve(pps):
    class DictPSO(pps.PSOAlgorithm):
        def pso_solve(self, prob, *, maxiters, **kwargs):
            pts = [prob.u0 + k for k in range(3)]
            return {"position": pts[1], "cost": 0.0}, [{"position": q} for q in pts], 1.25

    prob = pps.OptimizationProblem(lambda u, p: float(u.sum()), [0.0, 1.0])
    gbest, particles, t = pps.pso_solve(prob, DictPSO(), maxiters=5)
    assert t == 1.25 and len(particles) == 3
    sol = pps.solve(prob, DictPSO())
    assert np.array_equal(sol.u, [1.0, 2.0]) and sol.objective == 3.0
    assert [list(q) for q in sol.original] == [[0, 1], [1, 2], [2, 3]]
    assert sol.stats.time == 1.25


def test_an_algorithm_without_pso_solve_says_so(pps):
    class Bare(pps.PSOAlgorithm):
        pass

    prob = pps.OptimizationProblem(lambda u, p: 0.0, [0.0])
    with pytest.raises(NotImplementedError, match="Bare"):
        pps.solve(prob, Bare())
    with pytest.raises(pps.ArgumentError):
        pps.init(prob, Bare())


def test_device_objective_needs_the_device(pps):
    """With one of the engine's objectives, f(u, p) is computed by the library on
    the GPU; without one the call fails loudly instead of falling back."""
    import ctypes

    from parallelparticleswarms import _lib

    n = ctypes.c_int32(-1)
    if _lib.load().pps_device_count(ctypes.byref(n)) == _lib.OK and n.value > 0:
        pytest.skip("a CUDA device is present")
    prob = pps.OptimizationProblem(pps.sphere, [1.0, -2.0])
    with pytest.raises(pps.PPSError):
        pps.solve(prob, _u0_algorithm(pps))


def _u0_algorithm(pps):
    class U0(pps.PSOAlgorithm):
        def pso_solve(self, prob, *, maxiters, **kwargs):
            return Best(prob.u0.copy(), None), [Particle(prob.u0.copy())], 0.0

    return U0()


@pytest.mark.gpu
def test_device_objective_through_the_plugin(pps):
    sol = pps.solve(pps.OptimizationProblem(pps.sphere, [1.0, -2.0]), _u0_algorithm(pps))
    assert sol.objective == 5.0


def test_reference_cpu_algorithms_are_named_and_refused(pps):
    """ParallelPSOArray and SerialPSO (the reference's CPU algorithms) exist as
    names; solving with them says which GPU algorithm replaces them."""
    prob = pps.OptimizationProblem(pps.sphere, [1.0, -2.0], lb=[-5, -5], ub=[5, 5])
    for alg in (pps.ParallelPSOArray(100), pps.SerialPSO(100)):
        assert isinstance(alg, pps.PSOAlgorithm) and alg.num_particles == 100
        with pytest.raises(pps.PPSError, match="ParallelSyncPSOKernel") as e:
            pps.solve(prob, alg)
        assert e.value.code == 6  # PPS_ENOTSUP
