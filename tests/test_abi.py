"""The C ABI library: loads without a GPU, exports every symbol include/pps.h
declares, the Python binding covers them, and argument validation (host
logic, no device calls) behaves."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared(header="pps.h"):
    text = (ROOT / "include" / header).read_text()
    return sorted(set(re.findall(r"PPS_API\s+[\w\s\*]+?\b(pps_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared()
    for must in ("pps_swarm_create", "pps_swarm_init", "pps_sync_run", "pps_async_run", "pps_queue_run",
                 "pps_get_gbest", "pps_get_state", "pps_set_state", "pps_eval_objective", "pps_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(pps):
    from parallelparticleswarms import _lib

    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT\s+(pps_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    # nothing exported that the header does not declare
    assert exported <= set(declared()), sorted(exported - set(declared()))
    lib = _lib.load()
    for n in declared():
        assert hasattr(lib, n)
    assert set(_lib.declared_symbols()) == set(declared())


def test_version_and_error_without_gpu(pps):
    from parallelparticleswarms import _lib

    lib = _lib.load()
    assert lib.pps_version() == 100
    assert isinstance(lib.pps_last_error(), bytes)


def _prob(pps, **kw):
    args = dict(f=pps.rosenbrock, u0=np.zeros(3, np.float32), p=[1.0, 100.0], lb=np.full(3, -1.0, np.float32),
                ub=np.full(3, 10.0, np.float32))
    args.update(kw)
    return pps.OptimizationProblem(**args)


def test_argument_validation_precedes_device_use(pps):
    from parallelparticleswarms import _lib

    lib = _lib.load()
    h = ctypes.c_void_p()
    # dim 0
    pr = _prob(pps).to_c()
    pr.dim = 0
    assert lib.pps_swarm_create(ctypes.byref(pr), 10, 0, 0, ctypes.byref(h)) == _lib.EINVAL
    assert b"dim" in lib.pps_last_error()
    # lb > ub
    bad = _prob(pps, lb=np.full(3, 5.0, np.float32), ub=np.full(3, 1.0, np.float32)).to_c()
    assert lib.pps_swarm_create(ctypes.byref(bad), 10, 0, 0, ctypes.byref(h)) == _lib.EINVAL
    # NaN bound
    nanb = _prob(pps, lb=np.array([0, np.nan, 0], np.float32)).to_c()
    assert lib.pps_swarm_create(ctypes.byref(nanb), 10, 0, 0, ctypes.byref(h)) == _lib.EINVAL
    # unknown objective
    pr = _prob(pps).to_c()
    pr.objective = 99
    assert lib.pps_swarm_create(ctypes.byref(pr), 10, 0, 0, ctypes.byref(h)) == _lib.ENOTSUP
    # n = 0
    pr = _prob(pps).to_c()
    assert lib.pps_swarm_create(ctypes.byref(pr), 0, 0, 0, ctypes.byref(h)) == _lib.EINVAL
    # closed-form objective beyond its dimension
    pr = _prob(pps, f=pps.beale).to_c()
    assert lib.pps_swarm_create(ctypes.byref(pr), 10, 0, 0, ctypes.byref(h)) == _lib.EINVAL
    # NULL handles
    assert lib.pps_sync_run(None, 1, 0.7, 1.0, 1.4, 1.4, None) == _lib.EINVAL
    assert lib.pps_get_gbest(None, None, None, None) == _lib.EINVAL


def test_python_layer_rejects_other_backends(pps):
    with pytest.raises(pps.ArgumentError):
        pps.ParallelSyncPSOKernel(10, backend="cpu")
    with pytest.raises(pps.ArgumentError):
        pps.ParallelPSOKernel(0)
    # a Python callable is a problem only for a pso_solve algorithm: every
    # device path refuses it before touching the device
    prob = pps.OptimizationProblem(lambda x, p: 0.0, np.zeros(2))
    with pytest.raises(pps.ArgumentError, match="callable"):
        pps.init(prob, pps.ParallelSyncPSOKernel(10))
    with pytest.raises(pps.ArgumentError, match="callable"):
        pps.solve(prob, pps.HybridPSO(pps.ParallelPSOKernel(10)))
    with pytest.raises(pps.ArgumentError, match="callable"):
        pps.evaluate(prob, np.zeros(2))
    with pytest.raises(pps.ArgumentError, match="callable"):
        pps.Swarm(prob, 10)
    with pytest.raises(pps.ArgumentError):
        pps.OptimizationProblem(42, np.zeros(2))
