"""User objectives on the CPU: the oracle's C build of a user source agrees
bit for bit with the registered objectives it restates, a swarm over it runs
the registered swarm's iterations, and the library compiles sources with
NVRTC (no GPU needed) and reports compile errors with the compiler's log."""
import numpy as np
import pytest

import user_sources as us


def _points(D, n, lo, hi, seed):
    return np.random.default_rng(seed).uniform(lo, hi, (n, D)).astype(np.float32)


@pytest.mark.parametrize("src,obj,D,params", [
    (us.ROSENBROCK, 1, 7, [1.0, 100.0]),
    (us.RASTRIGIN, 2, 33, [10.0]),
    (us.SHIFTED_SPHERE, 7, 5, [2.0, 1.0, -0.5]),
])
def test_user_source_matches_registered_objective(orc, src, obj, D, params):
    user = orc.UserObjective(src)
    reg = orc.OracleProblem(obj, D, params=params)
    for x in _points(D, 500, -5.12, 5.12, seed=D):
        want = np.float32(reg.objective(x))
        got = np.float32(user(x, params))
        assert got == want or (np.isnan(got) and np.isnan(want)), (x, got, want)


def test_user_swarm_runs_the_registered_iterations(orc):
    D, n = 3, 300
    lb, ub = np.full(D, -1, np.float32), np.full(D, 10, np.float32)
    user = orc.UserObjective(us.ROSENBROCK)
    a = orc.OracleSwarm(orc.OracleProblem(1, D, lb, ub, params=[1.0, 100.0]), n, 4).init()
    b = orc.OracleSwarm(orc.OracleProblem(0, D, lb, ub, params=[1.0, 100.0], user=user), n, 4).init()
    a.sync_run(25)
    b.sync_run(25)
    for k in ("x", "v", "pbest", "pcost", "cost"):
        assert np.array_equal(a.state()[k], b.state()[k]), k
    assert a.gidx == b.gidx


def test_user_data_objective_on_the_oracle(orc):
    t = np.linspace(-1, 1, 40, dtype=np.float32)
    y = (0.5 - 2.0 * t + 3.0 * t * t).astype(np.float32)
    data = np.concatenate([t, y])
    user = orc.UserObjective(us.POLYFIT)
    assert user([0.5, -2.0, 3.0], data=data) < 1e-12
    assert user([0.0, 0.0, 0.0], data=data) > 1.0


def _register(pps, src):
    try:
        return pps.cuda_objective(src)
    except pps.PPSError as e:
        if e.code == 6:  # PPS_ENOTSUP: no NVRTC on this machine
            pytest.skip(str(e))
        raise


def test_register_compiles_and_deduplicates(pps):
    pkg = pps
    a = _register(pkg, us.ROSENBROCK)
    b = _register(pkg, us.ROSENBROCK)
    c = _register(pkg, us.RASTRIGIN)
    assert a.id == b.id >= 256 and c.id != a.id
    assert a.source == us.ROSENBROCK


def test_register_reports_compile_errors(pps):
    pkg = pps
    _register(pkg, us.SHIFTED_SPHERE)  # skips without NVRTC
    with pytest.raises(pkg.ArgumentError) as e:
        pkg.cuda_objective(us.HEAD + " { return undefined_name; }")
    assert "objective(1)" in str(e.value) and "undefined_name" in str(e.value)
    with pytest.raises(pkg.ArgumentError):
        pkg.cuda_objective("")


def test_register_with_gradient_compiles_the_local_stage(pps):
    """A source with PPS_HAS_GRADIENT compiles the HybridPSO local-stage
    kernels too (the shared device code of pps_local.cuh under NVRTC), and
    the oracle's C build of it has the gradient of the registered Rosenbrock."""
    pkg = pps
    f = _register(pkg, us.ROSENBROCK_GRAD)
    assert f.id >= 256


def test_user_gradient_on_the_oracle(orc):
    user = orc.UserObjective(us.ROSENBROCK_GRAD)
    assert user.grad is not None and orc.UserObjective(us.ROSENBROCK).grad is None
    reg = orc.OracleProblem(1, 12, params=[1.0, 100.0])
    usr = orc.OracleProblem(0, 12, params=[1.0, 100.0], user=user)
    for x in _points(12, 200, -3.0, 3.0, seed=5):
        fa, ga = reg.objective_grad(x)
        fb, gb = usr.objective_grad(x)
        assert np.float32(fa) == np.float32(fb) and np.array_equal(ga, gb)


@pytest.mark.parametrize("name,D,params,data", [
    ("RASTRIGIN_STREAM", 33, [10.0], None),
    ("ROSENBROCK_STREAM", 7, [1.0, 100.0], None),
    ("ROSENBROCK_STREAM", 1, [1.0, 100.0], None),
    ("SHIFTED_SPHERE_STREAM", 11, [2.0, 1.0, -0.5], None),
    ("WEIGHTED_SPHERE_STREAM", 9, [], np.linspace(0.5, 4.5, 9, dtype=np.float32)),
])
def test_stream_fold_equals_the_objective(orc, name, D, params, data):
    """The contract of PPS_HAS_STREAM on the test sources: the fold the step
    kernel drives (start, add in increasing d, finish) equals pps_objective bit
    for bit, NaN and Inf inputs included, and the objective part is the
    source it extends."""
    user = orc.UserObjective(getattr(us, name))
    assert user.stream_fn is not None and orc.UserObjective(us.RASTRIGIN).stream_fn is None
    pts = list(_points(D, 400, -6.0, 6.0, seed=D + 1))
    pts += [np.full(D, v, np.float32) for v in (0.0, -0.0, 1e30, np.inf, np.nan)]
    for x in pts:
        want, got = np.float32(user(x, params, data)), np.float32(user.stream(x, params, data))
        assert got.tobytes() == want.tobytes() or (np.isnan(got) and np.isnan(want)), (name, x, got, want)
    base = name.replace("_STREAM", "")
    if hasattr(us, base):
        plain = orc.UserObjective(getattr(us, base))
        for x in pts[:50]:
            assert np.float32(plain(x, params, data)).tobytes() == np.float32(user(x, params, data)).tobytes()


def test_register_with_stream_compiles(pps):
    """NVRTC compiles the step kernels' fold for PPS_HAS_STREAM sources, and a
    source that declares the macro without the functions is a compile error."""
    pkg = pps
    ids = {_register(pkg, getattr(us, n)).id for n in ("RASTRIGIN_STREAM", "ROSENBROCK_STREAM",
                                                          "SHIFTED_SPHERE_STREAM", "WEIGHTED_SPHERE_STREAM")}
    assert len(ids) == 4 and min(ids) >= 256
    with pytest.raises(pkg.ArgumentError) as e:
        pkg.cuda_objective("#define PPS_HAS_STREAM 1\n" + us.SHIFTED_SPHERE)
    assert "pps_stream" in str(e.value)
