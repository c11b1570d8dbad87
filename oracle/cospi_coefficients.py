"""The polynomial of cos(2 pi x) in the kernels and the oracle -- TEST INFRASTRUCTURE.

cos(pi a) for 0 <= a <= 1/2 is written (1/4 - a^2) Q(a^2) with
Q(z) = cos(pi sqrt z) / (1/4 - z), smooth on [0, 1/4] (the zero at a = 1/2 is
factored out) and Q(0) = 4 exactly, so Q(z) = 4 + z P(z).  P is the degree-3
polynomial minimising the maximum relative error of Q, fitted by iteratively
reweighted least squares (Lawson's algorithm) on Chebyshev nodes.  Run as a
script to print the binary32 coefficients the kernels (pps_device.cuh
kCosP0..3) and the oracle (pps_oracle.c COS_P0..3) compile.
"""
from __future__ import annotations

import numpy as np

COMPILED = ["-0x1.de9e60p+1", "0x1.472a8ap+0", "-0x1.d47d94p-3", "0x1.8c391ap-6"]


def q_true(z: np.ndarray) -> np.ndarray:
    a = np.sqrt(z)
    d = 0.5 - a
    out = np.empty_like(z)
    m = d > 1e-4
    out[m] = np.cos(np.pi * a[m]) / (0.25 - z[m])
    dd = d[~m]  # sin(pi d) / (d (1/2 + a)) near the removable singularity
    out[~m] = np.pi * (1 - (np.pi * dd) ** 2 / 6 + (np.pi * dd) ** 4 / 120) / (0.5 + a[~m])
    return out


def fit(degree: int = 3, nodes: int = 6000, iters: int = 200) -> np.ndarray:
    s = 0.5 - 0.5 * np.cos(np.pi * (np.arange(nodes) + 0.5) / nodes)  # Chebyshev nodes, s = 4 z in [0, 1]
    z = s / 4
    f = q_true(z)
    V = np.vander(s, degree + 1, increasing=True) * z[:, None]
    g = f - 4.0
    w = 1 / np.abs(f)
    for _ in range(iters):
        c, *_ = np.linalg.lstsq(V * w[:, None], g * w, rcond=None)
        err = (V @ c - g) / f
        w = w * np.sqrt(np.abs(err) + 1e-300)
        w /= w.max()
    return c * 4.0 ** np.arange(degree + 1)  # coefficients in z


def max_rel_error(coef) -> float:
    z = np.linspace(0, 0.25, 400001)
    q = 4 + z * (np.vander(z, len(coef), increasing=True) @ np.asarray(coef, np.float64))
    return float(np.abs((q - q_true(z)) / q_true(z)).max())


if __name__ == "__main__":
    c = fit()
    print("fitted:", [float(np.float32(v)).hex() for v in c], "max rel error", max_rel_error(c))
    print("compiled:", COMPILED, "max rel error", max_rel_error([float.fromhex(h) for h in COMPILED]))
