"""The rational tanh that the MLP kernel evaluates on the FMA pipe (pps_mlp.cu tanh_fma).

Why: the MLP objective needs one tanh per sample, particle and hidden unit.
tanh.approx.f32 runs on the special-function pipe at 16 per clock per SM,
while the FP32 pipe does 128 operations per clock per SM and sits mostly
idle, so part of the hidden units go through this approximation instead.

Method:
  - tanh is odd, so on |x| <= C it is approximated by a rational function
    x P(x^2) / Q(x^2), P of degree 2 and Q of degree 3 with Q(0) = 1, fitted
    for the least maximum absolute error by Loeb's linearisation with Lawson's
    iterative reweighting on a dense grid;
  - beyond C the argument is clamped, giving +-tanh(C): C is chosen so that
    1 - tanh(C) is about the fit's error;
  - 1 / Q is computed without the special-function pipe: a seed from the
    bits, y0 = float(R - bits(Q)), refined by one Newton step
    y1 = y0 + y0 e0 (e0 = 1 - Q y0) and one third-order step
    y2 = y1 + y1 (e1 + e1^2); R minimises the seed's maximum relative error.
Run as a script to print the binary32 constants and the maximum error of the
binary32 evaluation; COMPILED holds what pps_mlp.cu compiles.
"""
from __future__ import annotations

import numpy as np

# kTanhClamp, kTanhA0..A2, kTanhB1..B3, kRcpMagic as compiled in pps_mlp.cu
COMPILED = {
    "C": "0x1.900000p+2",
    "A": ["0x1.fffb1ep-1", "0x1.d2ccf0p-4", "0x1.7fcdecp-10"],
    "B": ["0x1.c9ea3ep-2", "0x1.1b6c34p-6", "0x1.be8a44p-15"],
    "R": 0x7EF311C2,
}


def fit(C: float, m: int = 3, k: int = 3, grid: int = 40000, iters: int = 80):
    x = np.linspace(0.0, C, grid)[1:]
    t = np.tanh(x)
    z = x * x
    A = np.hstack([np.stack([x * z ** i for i in range(m)], 1), np.stack([-t * z ** i for i in range(1, k + 1)], 1)])
    w = np.ones_like(x)
    q = np.ones_like(x)
    best = None
    for _ in range(iters):
        W = np.sqrt(w) / q
        sol, *_ = np.linalg.lstsq(A * W[:, None], t * W, rcond=None)
        a, b = sol[:m], sol[m:]
        P = x * sum(a[i] * z ** i for i in range(m))
        Q = 1.0 + sum(b[i] * z ** (i + 1) for i in range(k))
        e = P / Q - t
        err = float(np.max(np.abs(e)))
        if best is None or err < best[0]:
            best = (err, a.copy(), b.copy())
        q = Q
        w = w * np.abs(e)
        w = w / w.sum()
    return best


def rcp_magic() -> int:
    """R minimising max |1 - q float(R - bits(q))| over q in [1, 2)."""
    q = np.linspace(1.0, 2.0, 1 << 16, endpoint=False).astype(np.float32)
    qi = q.view(np.uint32).astype(np.int64)

    def worst(R):
        y = (R - qi).astype(np.uint32).view(np.float32).astype(np.float64)
        return float(np.max(np.abs(1.0 - q.astype(np.float64) * y)))

    lo, hi = 0x7EE00000, 0x7F000000
    for _ in range(60):  # ternary search: the error is unimodal in R
        m1, m2 = lo + (hi - lo) // 3, hi - (hi - lo) // 3
        if worst(m1) < worst(m2):
            hi = m2
        else:
            lo = m1
        if hi - lo < 3:
            break
    return min(range(lo, hi + 1), key=worst)


def _fma(a, b, c):
    """binary32 fused multiply-add (the float64 product of two binary32 values is exact)."""
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(np.float32)


def tanh_fma(h, C, A, B, R):
    """The kernel's sequence of binary32 operations."""
    f32 = np.float32
    x = np.minimum(np.maximum(np.asarray(h, np.float32), f32(-C)), f32(C))
    z = (x * x).astype(np.float32)
    p = _fma(f32(A[2]), z, f32(A[1]))
    p = _fma(p, z, f32(A[0]))
    p = (p * x).astype(np.float32)
    q = _fma(f32(B[2]), z, f32(B[1]))
    q = _fma(q, z, f32(B[0]))
    q = _fma(q, z, f32(1.0))
    y = (np.int64(R) - q.view(np.uint32).astype(np.int64)).astype(np.uint32).view(np.float32)
    e = _fma(-q, y, f32(1.0))
    y = _fma(y, e, y)
    e = _fma(-q, y, f32(1.0))
    y = _fma(y, _fma(e, e, e), y)
    return (p * y).astype(np.float32)


def compiled():
    C = float.fromhex(COMPILED["C"])
    A = [float.fromhex(v) for v in COMPILED["A"]]
    B = [float.fromhex(v) for v in COMPILED["B"]]
    return C, A, B, COMPILED["R"]


def max_abs_error(C, A, B, R, n: int = 2_000_001) -> float:
    h = np.linspace(-12.0, 12.0, n).astype(np.float32)
    return float(np.max(np.abs(tanh_fma(h, C, A, B, R).astype(np.float64) - np.tanh(h.astype(np.float64)))))


if __name__ == "__main__":
    C = 6.25
    err, a, b = fit(C)
    A = [float(np.float32(v)) for v in a]
    B = [float(np.float32(v)) for v in b]
    R = rcp_magic()
    print(f"fit on [0, {C}]: max error {err:.3e}, 1 - tanh(C) = {1 - np.tanh(C):.3e}")
    print("C", float(np.float32(C)).hex(), "A", [v.hex() for v in A], "B", [v.hex() for v in B], "R", hex(R))
    print("binary32 evaluation: max |error| over [-12, 12]", f"{max_abs_error(C, A, B, R):.3e}")
    print("compiled: max |error|", f"{max_abs_error(*compiled()):.3e}")
