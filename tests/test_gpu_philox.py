"""The device random stream and math functions against independent
implementations: cuRAND's Philox4_32_10 generator (run, not read) and the
oracle's C restatement; cos/sin/exp against float64 numpy."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def checklib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = tmp_path_factory.mktemp("philox") / "philox_check.so"
    subprocess.run([nvcc, "-shared", "-Xcompiler", "-fPIC", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                    "-fmad=false", "-std=c++17", f"-I{ROOT / 'parallelparticleswarms.jl_gb300' / 'csrc'}",
                    f"-I{ROOT / 'include'}", "-o", str(out), str(ROOT / "tests" / "cuda" / "philox_check.cu")],
                   check=True)
    lib = ctypes.CDLL(str(out))
    return lib


def test_device_philox_matches_oracle_and_curand(checklib, orc):
    rng = np.random.default_rng(0)
    n = 4096
    ck = rng.integers(0, 2**32, size=(n, 6), dtype=np.uint64).astype(np.uint32)
    ck[:, 1] = 0          # cuRAND's offset only reaches counter word 0
    ck[:, 0] %= 1 << 20
    ck[:8] = 0
    ck[1, 4] = 1
    ck = np.ascontiguousarray(ck)
    ours = np.zeros((n, 4), np.uint32)
    theirs = np.zeros((n, 4), np.uint32)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    rc = checklib.philox_check(n, ck.ctypes.data_as(u32p), ours.ctypes.data_as(u32p), theirs.ctypes.data_as(u32p))
    assert rc == 0
    ref = np.array([orc.philox4x32_10(list(map(int, c[:4])), list(map(int, c[4:]))) for c in ck], np.uint32)
    assert np.array_equal(ours, ref), "device Philox differs from the oracle"
    # cuRAND: state(seed=key, subsequence=ctr.zw, offset=4*ctr.x) yields philox(ctr, key) first
    assert np.array_equal(theirs, ref), f"{np.mean(np.all(theirs == ref, axis=1)):.3f} of blocks agree with cuRAND"


def test_device_math_matches_oracle_bitwise(checklib, orc):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-6, 6, 50000), rng.uniform(-90, 90, 20000), rng.uniform(-1e4, 1e4, 5000),
                        np.array([0.0, -0.0, 0.25, 0.5, 0.75, 1.0, np.inf, -np.inf, np.nan, 1e-30, 88.7, -87.3])
                        ]).astype(np.float32)
    n = x.size
    out = np.zeros((n, 4), np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    assert checklib.math_check(n, x.ctypes.data_as(fp), out.ctypes.data_as(fp)) == 0
    L = orc.load()
    c = np.array([L.orc_cos2pi(float(v)) for v in x], np.float32)
    s = np.array([L.orc_sin2pi(float(v)) for v in x], np.float32)
    e = np.array([L.orc_exp(float(v)) for v in x], np.float32)
    u = np.array([L.orc_u01(int(b)) for b in x.view(np.uint32)], np.float32)
    assert np.array_equal(out[:, 0], c, equal_nan=True)
    assert np.array_equal(out[:, 1], s, equal_nan=True)
    assert np.array_equal(out[:, 2], e, equal_nan=True)
    assert np.array_equal(out[:, 3], u)
