"""The FP32-pipe tanh of the MLP kernel (pps_mlp.cu tanh_fma), on the CPU:
its constants are the ones tanh_coefficients.py fits, and its binary32
sequence of operations (emulated in numpy) stays within 2e-5 of tanh over
all finite inputs, well inside the special-function tanh.approx.f32's
relative error of about 2^-11 that it stands in for."""
import re
import sys
from pathlib import Path

import numpy as np

CSRC = Path(__file__).resolve().parent.parent / "parallelparticleswarms.jl_gb300" / "csrc"


def _tc():
    sys.path.insert(0, str(CSRC))
    try:
        import tanh_coefficients as tc
    finally:
        sys.path.pop(0)
    return tc


def test_kernel_compiles_the_fitted_constants():
    tc = _tc()
    src = (CSRC / "pps_mlp.cu").read_text()
    C, A, B, R = tc.compiled()

    def const(name):
        m = re.search(name + r" = (0x[0-9a-fA-Fp.+-]+)f", src)
        assert m, name
        return float.fromhex(m.group(1))

    assert const("kTanhClamp") == C
    assert [const(f"kTanhA{k}") for k in range(3)] == A
    assert [const(f"kTanhB{k}") for k in range(1, 4)] == B
    assert int(re.search(r"kRcpMagic = (0x[0-9A-Fa-f]+);", src).group(1), 16) == R


def test_fit_reproduces_the_compiled_constants():
    tc = _tc()
    err, a, b = tc.fit(float.fromhex(tc.COMPILED["C"]))
    assert [float(np.float32(v)).hex() for v in a] == [float.fromhex(h).hex() for h in tc.COMPILED["A"]]
    assert [float(np.float32(v)).hex() for v in b] == [float.fromhex(h).hex() for h in tc.COMPILED["B"]]
    assert tc.rcp_magic() == tc.COMPILED["R"]


def test_binary32_error_bound():
    tc = _tc()
    assert tc.max_abs_error(*tc.compiled()) < 2e-5
    C, A, B, R = tc.compiled()
    # odd, saturating, and exact signs at the extremes
    h = np.array([0.0, -0.0, 1e-30, -1e-30, 1e30, -1e30, np.finfo(np.float32).max], np.float32)
    t = tc.tanh_fma(h, C, A, B, R)
    assert t[0] == 0.0 and t[2] > 0 and t[3] < 0 and abs(t[4] - 1) < 2e-5 and abs(t[5] + 1) < 2e-5
    x = np.linspace(0, 8, 10001).astype(np.float32)
    assert np.array_equal(tc.tanh_fma(-x, C, A, B, R), -tc.tanh_fma(x, C, A, B, R))
