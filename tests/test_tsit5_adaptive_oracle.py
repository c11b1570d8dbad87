"""Adaptive Tsit5 for ode_pso (parameter_estim_ode!(..., Val(true)),
src/ode_pso.jl:54-111) in the oracle, on the CPU.

The reference hands adaptive integration to DiffEqGPU's vectorized_asolve
(not vendored).  This build restates the published pieces: the embedded
4th-order error estimate of Tsitouras' pair and the PI step-size controller
of Hairer, Norsett & Wanner (Solving ODEs I, sec. II.4).  Checked here:

  - the compiled error weights d = b - bhat are the derived ones: bhat meets
    every order-4 condition, misses an order-5 one (a genuine lower-order
    companion), and is the minimum-norm member of the one-parameter family
    those conditions leave; the CUDA header and the oracle compile the same
    binary32 values;
  - the controller's own ln x (orc_log, the kernels' log_f) within 2.5e-7
    relative of ln over the positive binary32 range;
  - on the reference's LV and FHN benchmark problems the adaptive solution
    converges to an accurate one as the tolerance tightens, with more steps;
  - an unreachable tolerance ends with a loss of +inf, bounded in steps;
  - the C ABI rejects bad tolerances before any device use."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import tsit5_coefficients as tc

ROOT = Path(__file__).resolve().parent.parent


def test_error_weights_are_the_derived_ones():
    d = tc.derive_embedded()
    assert [float(np.float32(v)).hex() for v in d] == [float.fromhex(h).hex() for h in tc.LITERALS_D]
    bhat = tc.B - d
    M, r = tc.order4_conditions()
    assert np.abs(M @ bhat - r).max() < 1e-12
    c = tc.C
    assert abs(bhat @ c ** 4 - 1 / 5) > 1e-3  # not an order-5 solution
    # minimum norm within the family bhat + s n (n spanning the conditions' null space)
    n = np.linalg.svd(M)[2][-1]
    assert abs(bhat @ n) < 1e-12
    want = [float.fromhex(h) for h in tc.LITERALS_D]
    cu = (ROOT / "parallelparticleswarms.jl_gb300" / "csrc" / "pps_ode.cuh").read_text()
    got_cu = [float.fromhex(v) for v in re.findall(r"\bd\d = (-?0x[0-9a-f.]+p[+-]\d+)f", cu)]
    assert got_cu == want
    orc_src = (ROOT / "oracle" / "pps_oracle_ode.c").read_text()
    block = orc_src[orc_src.index("D_ERR[7]"):orc_src.index("};", orc_src.index("D_ERR[7]"))]
    assert [float.fromhex(v) for v in re.findall(r"(-?0x[0-9a-f.]+p[+-]\d+)f", block)] == want


def test_controller_log(orc):
    L = orc.load()
    xs = np.concatenate([np.geomspace(1e-45, 3e38, 40001), np.linspace(0.5, 2.0, 20001),
                         [np.float32(1.0), np.nextafter(np.float32(1), np.float32(2))]]).astype(np.float32)
    xs = xs[xs > 0]
    got = np.array([L.orc_log(float(x)) for x in xs], np.float64)
    want = np.log(xs.astype(np.float64))
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-7)) < 2.5e-7
    assert L.orc_log(1.0) == 0.0 and L.orc_log(0.0) == -np.inf and np.isnan(L.orc_log(-1.0))
    assert L.orc_log(float("inf")) == np.inf


def _dense64(model, p, u0, t, l=0.0, h=1e-4):
    """float64 RK4 at step h sampled at t (multiples of h): the accurate solution."""
    def f(u):
        if model == "lv":
            return np.array([p[0] * u[0] - p[1] * u[0] * u[1], -p[2] * u[1] + p[3] * u[0] * u[1]])
        return np.array([u[0] - u[0] ** 3 / 3 - u[1] + l, p[2] * (u[0] + p[0] - p[1] * u[1])])
    u = np.array(u0, np.float64)
    out, s = [], 0
    for m in np.rint(np.asarray(t) / h).astype(int):
        while s < m:
            k1 = f(u)
            k2 = f(u + h / 2 * k1)
            k3 = f(u + h / 2 * k2)
            k4 = f(u + h * k3)
            u = u + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
            s += 1
        out.append(u.copy())
    return np.array(out)


@pytest.mark.parametrize("model", ["lv", "fhn"])
def test_adaptive_solution_converges(pps, orc, model):
    from parallelparticleswarms import ode

    prob, truth = ode.reference_benchmark_fit(model)
    t = np.arange(prob.data.size // 2) * 0.01
    l = float(truth[3]) if model == "fhn" else 0.0
    exact = _dense64(model, truth[:4] if model == "lv" else truth[:3], (1.0, 1.0), t, l=l)
    errs, steps = [], []
    for rt in (1e-3, 1e-4, 1e-5, 1e-6):
        op = orc.ode_fit_problem(ode.adaptive(prob, reltol=rt, abstol=rt * 1e-3))
        sol = op.ode.solve(truth.astype(np.float32))
        _, n = op.ode.loss_adaptive(truth.astype(np.float32))
        errs.append(float(np.max(np.abs(sol - exact))))
        steps.append(n)
    assert all(np.isfinite(errs))
    assert errs[-1] < errs[0] and errs[-1] < 1e-4, errs
    assert steps == sorted(steps) and steps[0] < steps[-1], steps
    assert errs[0] < 50 * 1e-3, errs  # the loosest tolerance still tracks the solution


def test_unreachable_tolerance_gives_inf_within_the_step_bound(pps, orc):
    from parallelparticleswarms import ode

    prob, truth = ode.reference_benchmark_fit("lv")
    op = orc.ode_fit_problem(ode.adaptive(prob, reltol=1e-30, abstol=1e-38))
    f, n = op.ode.loss_adaptive(truth.astype(np.float32))
    assert f == np.inf and n <= 100000


def test_abi_rejects_bad_tolerances(pps):
    from parallelparticleswarms import _lib, ode

    lib = _lib.load()
    prob, _ = ode.reference_benchmark_fit("lv")
    for rt, at, dt in ((0.0, 1e-6, 0.1), (1e-3, -1.0, 0.1), (float("nan"), 1e-6, 0.1), (1e-3, 1e-6, 0.0),
                       (1e-3, float("inf"), 0.1)):
        p = ode.adaptive(prob, reltol=1e-3, abstol=1e-6)
        p.p[2], p.p[3], p.p[4] = dt, rt, at
        pr = p.to_c()
        h = ctypes.c_void_p()
        assert lib.pps_swarm_create(ctypes.byref(pr), 16, 0, 0, ctypes.byref(h)) == _lib.EINVAL
        assert b"adaptive" in lib.pps_last_error()
