"""Argument validation of the later C-ABI entry points, on the host and
without a GPU: ODE fit options (RK4 / Tsit5), user-objective registration and
ids, particle records and position snapshots.  Every case returns its status
before the library touches a device."""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib(pps):
    from parallelparticleswarms import _lib

    return _lib.load()


def _create(lib, prob, n=16):
    from parallelparticleswarms import _lib

    h = ctypes.c_void_p()
    pr = prob.to_c()
    rc = lib.pps_swarm_create(ctypes.byref(pr), n, 0, 0, ctypes.byref(h))
    assert h.value is None, "a rejected problem leaves no swarm behind"
    return rc, lib.pps_last_error().decode(), _lib


def _lv(pps, nsaves=11, **kw):
    data = np.ones(2 * nsaves, np.float32)
    return pps.ode.lv_problem(data, dt=0.01, nsteps=100, save_every=10, **kw)


def test_ode_method_and_save_spacing(pps, lib):
    # an unknown integrator id in params[6] (0 RK4, 1 Tsit5, 2 adaptive Tsit5)
    prob = _lv(pps, method="tsit5", save_dt=0.1)
    prob.p[6] = 3.0
    rc, msg, L = _create(lib, prob)
    assert rc == L.EINVAL and "method" in msg
    # Tsit5 without a positive, finite save spacing
    for bad in (0.0, -0.1, np.inf, np.nan):
        prob = _lv(pps, method="tsit5", save_dt=0.1)
        prob.p[7] = bad
        rc, msg, L = _create(lib, prob)
        assert rc == L.EINVAL and "save_dt" in msg, bad
    # Tsit5 observations beyond the integrated span: 10 * 0.2 > 100 * 0.01
    rc, msg, L = _create(lib, _lv(pps, method="tsit5", save_dt=0.2))
    assert rc == L.EINVAL and "exceeds" in msg
    # RK4 observations beyond the integrated span: 20 saves every 10 of 100 steps
    rc, msg, L = _create(lib, _lv(pps, nsaves=21))
    assert rc == L.EINVAL and "exceeds" in msg


def test_ode_model_shapes(pps, lib):
    # the Lotka-Volterra fit has exactly 4 parameters
    prob = _lv(pps)
    prob.dim = 3
    rc, msg, L = _create(lib, prob)
    assert rc == L.EINVAL and "4 parameters" in msg
    # FitzHugh-Nagumo takes 3 or 4 (with l)
    data = np.ones(22, np.float32)
    prob = pps.ode.fhn_problem(data, dt=0.01, nsteps=100, save_every=10, fit_l=True)
    prob.dim = 2
    rc, msg, L = _create(lib, prob)
    assert rc == L.EINVAL and "FitzHugh-Nagumo" in msg
    prob.dim = 5
    rc, msg, L = _create(lib, prob)
    assert rc == L.EINVAL and "at most 4 parameters" in msg
    # observations come as (u1, u2) pairs
    prob = _lv(pps)
    prob.data = np.ones(21, np.float32)
    rc, msg, L = _create(lib, prob)
    assert rc == L.EINVAL and "2 * nsaves" in msg
    # non-integral step counts
    prob = _lv(pps)
    prob.p[3] = 100.5
    rc, msg, L = _create(lib, prob)
    assert rc == L.EINVAL and "integral" in msg


def test_python_ode_options(pps):
    data = np.ones(22, np.float32)
    with pytest.raises(ValueError, match="save_dt"):
        pps.ode.lv_problem(data, method="tsit5")
    with pytest.raises(ValueError, match="method"):
        pps.ode.fhn_problem(data, method="euler")


def test_user_objective_registration_arguments(lib):
    from parallelparticleswarms import _lib

    oid = ctypes.c_int32(-1)
    assert lib.pps_objective_register(None, ctypes.byref(oid)) == _lib.EINVAL
    assert lib.pps_objective_register(b"", ctypes.byref(oid)) == _lib.EINVAL
    assert lib.pps_objective_register(b"PPS_DEVICE float x;", None) == _lib.EINVAL
    assert oid.value == -1


def test_unregistered_user_id_is_refused(pps, lib):
    # an id past the registered range is not an objective (no lookup past the table)
    from parallelparticleswarms import _lib

    prob = pps.OptimizationProblem(pps.sphere, np.zeros(3, np.float32), lb=np.full(3, -1.0, np.float32),
                                   ub=np.full(3, 1.0, np.float32))
    pr = prob.to_c()
    for oid in (256 + 4095, 256 + 4096, 1 << 30):
        pr.objective = oid
        h = ctypes.c_void_p()
        assert lib.pps_swarm_create(ctypes.byref(pr), 16, 0, 0, ctypes.byref(h)) == _lib.ENOTSUP
        x = np.zeros((3, 4), np.float32)
        f = np.zeros(4, np.float32)
        assert lib.pps_eval_objective(ctypes.byref(pr), 4, _lib.fptr(x), _lib.fptr(f)) == _lib.ENOTSUP


def test_records_and_snapshots_need_handles(lib):
    from parallelparticleswarms import _lib

    buf = np.zeros(16, np.float32)
    for layout in (_lib.LAYOUT_AOS, _lib.LAYOUT_SOA):
        assert lib.pps_get_particles(None, layout, _lib.fptr(buf)) == _lib.EINVAL
        assert lib.pps_set_particles(None, layout, _lib.fptr(buf)) == _lib.EINVAL
    c = ctypes.c_void_p()
    assert lib.pps_field_copy_create(None, 0, ctypes.byref(c)) == _lib.EINVAL
    assert lib.pps_field_copy_read(None, _lib.fptr(buf)) == _lib.EINVAL
    assert lib.pps_field_copy_destroy(None) == _lib.OK


def test_valid_calls_fail_loudly_without_a_device(pps, lib):
    """No CPU fallback: with no CUDA device every compute entry point says so."""
    from parallelparticleswarms import _lib

    n = ctypes.c_int32(-1)
    if lib.pps_device_count(ctypes.byref(n)) == _lib.OK and n.value > 0:
        pytest.skip("a CUDA device is present")
    prob = pps.OptimizationProblem(pps.sphere, np.zeros(3, np.float32), lb=np.full(3, -1.0, np.float32),
                                   ub=np.full(3, 1.0, np.float32))
    pr = prob.to_c()
    h = ctypes.c_void_p()
    assert lib.pps_swarm_create(ctypes.byref(pr), 16, 0, 0, ctypes.byref(h)) == _lib.ENODEV
    b = ctypes.c_void_p()
    assert lib.pps_batch_create(ctypes.byref(b)) == _lib.ENODEV
    x = np.zeros((3, 4), np.float32)
    f = np.zeros(4, np.float32)
    assert lib.pps_eval_objective(ctypes.byref(pr), 4, _lib.fptr(x), _lib.fptr(f)) == _lib.ENODEV
    with pytest.raises(pps.PPSError):
        pps.solve(prob, pps.ParallelSyncPSOKernel(16), maxiters=2)


def test_hybrid_refuses_tolerances_it_does_not_have(pps):
    from parallelparticleswarms.hybrid import hybrid_solve

    with pytest.raises(pps.ArgumentError, match="reltol"):
        hybrid_solve(None, reltol=1e-6)
    with pytest.raises(pps.ArgumentError, match="linesearch"):
        hybrid_solve(None, linesearch="strong_wolfe")


def test_standalone_bfgs_arguments(pps, monkeypatch):
    """solve(prob, BFGS()) (src/bfgs.jl:2-36): refuses what it does not have
    before any device work, defaults to 1000 iterations as the reference, and
    without a device fails loudly."""
    import parallelparticleswarms.hybrid as hy

    prob = pps.OptimizationProblem(pps.rosenbrock, [-1.2, 1.0], [1.0, 100.0])
    with pytest.raises(pps.ArgumentError, match="reltol"):
        pps.solve(prob, pps.BFGS(), reltol=1e-8)
    with pytest.raises(pps.ArgumentError, match="sampler"):
        pps.solve(prob, pps.BFGS(), sampler=pps.GPUUniformSampler())
    with pytest.raises(pps.ArgumentError, match="unexpected"):
        pps.solve(prob, pps.BFGS(), local_maxiters=3)
    seen = {}
    monkeypatch.setattr(hy, "bfgs_solve", lambda prob, alg, **kw: seen.update(kw) or "ran")
    assert pps.solve(prob, pps.BFGS()) == "ran" and seen["maxiters"] == 1000
    assert pps.solve(prob, pps.BFGS(), maxiters=7) == "ran" and seen["maxiters"] == 7
    monkeypatch.undo()
    from parallelparticleswarms import _lib

    n = ctypes.c_int32(-1)
    if _lib.load().pps_device_count(ctypes.byref(n)) == _lib.OK and n.value > 0:
        return
    with pytest.raises(pps.PPSError):
        pps.solve(prob, pps.BFGS())


def test_problem_limits(pps, lib):
    """The limits pps_swarm_create checks before it allocates anything."""
    from parallelparticleswarms import _lib

    def rc_of(pr, n=16):
        h = ctypes.c_void_p()
        rc = lib.pps_swarm_create(ctypes.byref(pr), n, 0, 0, ctypes.byref(h))
        assert h.value is None
        return rc, lib.pps_last_error().decode()

    base = pps.OptimizationProblem(pps.sphere, np.zeros(3, np.float32), lb=np.full(3, -1.0, np.float32),
                                   ub=np.full(3, 1.0, np.float32))
    assert rc_of(base.to_c(), n=(1 << 32))[0] == _lib.EINVAL          # n beyond 2^32 - 256
    big = pps.OptimizationProblem(pps.sphere, np.zeros(4097, np.float32))
    rc, msg = rc_of(big.to_c())
    assert rc == _lib.EINVAL and "dim" in msg
    p9 = pps.OptimizationProblem(pps.sphere, np.zeros(3, np.float32), np.ones(9, np.float32))
    rc, msg = rc_of(p9.to_c())
    assert rc == _lib.EINVAL and "nparams" in msg
    pr = base.to_c()
    pr.nparams = 2  # count without a pointer
    rc, msg = rc_of(pr)
    assert rc == _lib.EINVAL and "params" in msg
    row = pps.quadratic_constraint(3, c=-1.0, a=[1, 0, 0])
    five = base.remake(cons=np.stack([row] * 5))
    rc, msg = rc_of(five.to_c())
    assert rc == _lib.EINVAL and "ncons" in msg
    bad = row.copy()
    bad[2] = np.nan
    rc, msg = rc_of(base.remake(cons=bad[None, :]).to_c())
    assert rc == _lib.EINVAL and "finite" in msg


def test_serve_config_validation(lib):
    """pps_serve_start checks its configuration before it looks for a device;
    a valid one without a device is PPS_ENODEV."""
    from parallelparticleswarms import _lib

    h = ctypes.c_void_p()
    assert lib.pps_serve_start(None, None) == _lib.EINVAL
    for field, value in (("max_launches", 65), ("max_pack", 4097), ("threads", 96), ("ppt", 3)):
        cfg = _lib.ServeConfig()
        setattr(cfg, field, value)
        assert lib.pps_serve_start(ctypes.byref(cfg), ctypes.byref(h)) == _lib.EINVAL, field
        assert h.value is None
    n = ctypes.c_int32(-1)
    if lib.pps_device_count(ctypes.byref(n)) == _lib.OK and n.value > 0:
        return
    assert lib.pps_serve_start(ctypes.byref(_lib.ServeConfig()), ctypes.byref(h)) == _lib.ENODEV
    assert lib.pps_serve_stop(None) == _lib.OK
    assert lib.pps_serve_submit(None, None, 1, 0, 1, 0.7, 1.0, 1.4, 1.4, None) == _lib.EINVAL
