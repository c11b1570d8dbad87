"""Tsitouras' 5(4) pair and its continuous extension -- TEST INFRASTRUCTURE.

The reference integrates ode_pso with DiffEqGPU's GPUTsit5 (src/ode_pso.jl:58,
87,146; DiffEqGPU is not vendored).  GPUTsit5 is Tsitouras, "Runge-Kutta pairs
of order 5(4) satisfying only the first column simplifying assumption",
Computers & Mathematics with Applications 62 (2011) 770-775.  This script
holds that paper's tableau (the 7-stage FSAL pair: A's lower triangle and the
5th-order weights b = A's last row) and checks it against the 17 order-5
conditions; it then DERIVES the 4th-order continuous extension b_i(theta)
(theta = 0..1 across a step) from its conditions instead of quoting it:

  * b_i(theta) = delta_i1 theta + r_i2 theta^2 + r_i3 theta^3 + r_i4 theta^4;
  * the 8 order conditions up to order 4 hold for every theta;
  * b_i(1) = b_i, and b_i'(1) = delta_i7 (C1 at the step end: the FSAL stage);

which leave one free parameter, fixed by b_7(theta) = 1.5 theta^2 - 4 theta^3
+ 2.5 theta^4.  ``LITERALS`` are the decimal constants the oracle
(pps_oracle_ode.c) and the CUDA kernels (pps_ode.cuh) compile, rounded to
binary32 by the compilers; tests/test_tsit5_coefficients.py checks them
against this derivation.  Run as a script to print the derivation.
"""
from __future__ import annotations

import numpy as np

# Tsitouras (2011): stage i = 2..7 combines stages 1..i-1 with A[i-1, :i-1]
A = np.zeros((7, 7))
A[1, :1] = [0.161]
A[2, :2] = [-0.008480655492356989, 0.335480655492357]
A[3, :3] = [2.897153057105493, -6.359448489975075, 4.3622954328695815]
A[4, :4] = [5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525]
A[5, :5] = [5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383]
A[6, :6] = [0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081,
            2.324710524099774]
B = A[6].copy()  # first same as last: the 5th-order weights are stage 7's row, b_7 = 0
C = A.sum(axis=1)

# the interpolant's coefficients as compiled: R[i] = (r_i2, r_i3, r_i4); r_11 = 1
LITERALS_R = np.array([
    [-2.763706197274826, 2.9132554618219126, -1.0530884977290216],
    [0.1317, -0.2234, 0.1017],
    [3.9302962368947516, -5.941033872131505, 2.490627285651253],
    [-12.411077166933676, 30.33818863028232, -16.548102889244902],
    [37.50931341651104, -88.1789048947664, 47.37952196281928],
    [-27.896526289197286, 65.09189467479366, -34.87065786149661],
    [1.5, -4.0, 2.5],
])


# the error-estimate weights as compiled: d_i = b_i - bhat_i (i = 1..7), binary32
LITERALS_D = ["0x1.44f608p-7", "0x1.2a1940p-8", "-0x1.67af8ep-5", "0x1.9cca80p-1", "-0x1.9f4bdcp+1",
              "0x1.46ac0cp+1", "-0x1.59c28ep-4"]


def order4_conditions() -> tuple[np.ndarray, np.ndarray]:
    """Rows phi with rhs 1/gamma: the 8 order conditions up to order 4, as
    linear conditions on a weight vector."""
    c, Ac = C, A @ C
    trees = [(np.ones(7), 1), (c, 2), (c ** 2, 3), (Ac, 6), (c ** 3, 4), (c * Ac, 8), (A @ c ** 2, 12),
             (A @ Ac, 24)]
    return np.array([t for t, _ in trees]), np.array([1 / g for _, g in trees])


def derive_embedded() -> np.ndarray:
    """The embedded 4th-order weights bhat and the error weights d = b - bhat.

    On this pair's nodes the 8 order-4 conditions have rank 6 over the 7
    weights, so the embedded 4th-order solutions form a one-parameter family
    b + s n (n spans the null space; b itself satisfies them); every member
    gives an error estimate dt sum_i d_i k_i along the same direction, only
    its size changes with s.  This build takes the member of least Euclidean
    norm (the minimum-norm solution of the conditions), a choice of its own:
    DiffEqGPU's embedded weights are not vendored, so the adaptive step sizes
    are not pinned to the reference's."""
    M, r = order4_conditions()
    assert np.linalg.matrix_rank(M) == 6
    bhat = np.linalg.pinv(M) @ r
    assert np.abs(M @ bhat - r).max() < 1e-12
    return B - bhat


def order5_residuals() -> dict:
    b, c, Ac = B, C, A @ C
    t = {
        "1": (b.sum(), 1), "c": (b @ c, 1 / 2), "c2": (b @ c ** 2, 1 / 3), "Ac": (b @ Ac, 1 / 6),
        "c3": (b @ c ** 3, 1 / 4), "cAc": (b @ (c * Ac), 1 / 8), "Ac2": (b @ (A @ c ** 2), 1 / 12),
        "AAc": (b @ (A @ Ac), 1 / 24), "c4": (b @ c ** 4, 1 / 5), "c2Ac": (b @ (c ** 2 * Ac), 1 / 10),
        "cAc2": (b @ (c * (A @ c ** 2)), 1 / 15), "cAAc": (b @ (c * (A @ Ac)), 1 / 30),
        "(Ac)2": (b @ Ac ** 2, 1 / 20), "Ac3": (b @ (A @ c ** 3), 1 / 20), "AcAc": (b @ (A @ (c * Ac)), 1 / 40),
        "AAc2": (b @ (A @ (A @ c ** 2)), 1 / 60), "AAAc": (b @ (A @ (A @ Ac)), 1 / 120)}
    return {k: v - want for k, (v, want) in t.items()}


def derive_interpolant() -> np.ndarray:
    """Solve the continuous-extension conditions; returns R (7 x 3)."""
    c, Ac = C, A @ C
    trees = [(np.ones(7), 1, 1), (c, 2, 2), (c ** 2, 3, 3), (Ac, 3, 6), (c ** 3, 4, 4), (c * Ac, 4, 8),
             (A @ c ** 2, 4, 12), (A @ Ac, 4, 24)]
    rows, rhs = [], []

    def col(i, k):
        return 3 * i + (k - 2)
    for phi, rho, gamma in trees:  # theta^k coefficient of sum_i b_i(theta) phi_i = theta^rho / gamma
        for k in (2, 3, 4):
            row = np.zeros(21)
            for i in range(7):
                row[col(i, k)] = phi[i]
            rows.append(row)
            rhs.append(1 / gamma if k == rho else 0.0)
    for i in range(7):
        row = np.zeros(21)  # b_i(1) = b_i
        row[[col(i, 2), col(i, 3), col(i, 4)]] = 1
        rows.append(row)
        rhs.append(B[i] - (1.0 if i == 0 else 0.0))
        row = np.zeros(21)  # b_i'(1) = delta_i7
        row[[col(i, 2), col(i, 3), col(i, 4)]] = [2, 3, 4]
        rows.append(row)
        rhs.append((1.0 if i == 6 else 0.0) - (1.0 if i == 0 else 0.0))
    row = np.zeros(21)  # the free parameter: b_7(theta) = 1.5 theta^2 - ...
    row[col(6, 2)] = 1
    rows.append(row)
    rhs.append(1.5)
    M, y = np.array(rows), np.array(rhs)
    assert np.linalg.matrix_rank(M) == 21
    r, *_ = np.linalg.lstsq(M, y, rcond=None)
    assert np.abs(M @ r - y).max() < 1e-10
    return r.reshape(7, 3)


if __name__ == "__main__":
    res = order5_residuals()
    print("order-5 residuals: max", max(abs(v) for v in res.values()))
    R = derive_interpolant()
    np.set_printoptions(precision=16)
    print("derived interpolant (r_i2, r_i3, r_i4):\n", R)
    print("max |derived - literals|", np.abs(R - LITERALS_R).max())
    d = derive_embedded()
    print("error weights d = b - bhat (binary32):", [float(np.float32(v)).hex() for v in d])
