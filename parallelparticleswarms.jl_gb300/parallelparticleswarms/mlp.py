"""Training a small neural network by PSO (examples/neural_network/nn.jl).

The reference trains a SimpleChains MLP with ``ParallelPSOKernel(1000)``: the
particle is the flattened parameter vector and the objective the network's
loss on a data set (nn.jl:20-24 builds the chain, :52-62 the problem and the
solve).  Here the network is fixed by the engine's tensor-core kernel:

    16 inputs -> 32 tanh units -> 1 output, mean squared error over S samples

with the particle laid out as W1 (16 x 32, input-major: W1[i, j] at i*32 + j),
b1 (32), w2 (32), b2 (1): 577 parameters.  The samples enter the hidden-layer
GEMM as bfloat16 with float32 accumulation; S must be a multiple of 128
(one MMA block of samples) and at most 4096.

``teacher_task`` builds the data set of the workload on the host: Gaussian
inputs and the targets of a random teacher network of the same shape, so a
perfect fit exists.  It is input generation, not part of the solve.
"""
from __future__ import annotations

import numpy as np

from .problem import OptimizationProblem, mlp_regression

N_IN = 16
N_HIDDEN = 32
DIM = N_IN * N_HIDDEN + 2 * N_HIDDEN + 1  # 577


def pack(W1, b1, w2, b2) -> np.ndarray:
    """Flatten (W1 (16, 32), b1 (32,), w2 (32,), b2) into a 577-vector."""
    W1 = np.asarray(W1, np.float32).reshape(N_IN, N_HIDDEN)
    return np.concatenate([W1.reshape(-1), np.asarray(b1, np.float32).reshape(N_HIDDEN),
                           np.asarray(w2, np.float32).reshape(N_HIDDEN),
                           np.asarray(b2, np.float32).reshape(1)]).astype(np.float32)


def unpack(x):
    """The inverse of ``pack``: (W1 (16, 32), b1, w2, b2)."""
    x = np.asarray(x, np.float32).reshape(DIM)
    return (x[:N_IN * N_HIDDEN].reshape(N_IN, N_HIDDEN), x[512:544], x[544:576], float(x[576]))


def predict(x, X) -> np.ndarray:
    """Network output for inputs X (S, 16), float64 on the host (for inspection)."""
    W1, b1, w2, b2 = unpack(x)
    h = np.tanh(np.asarray(X, np.float64) @ W1.astype(np.float64) + b1)
    return h @ w2.astype(np.float64) + b2


def teacher_task(samples: int = 1024, seed: int = 0):
    """(data, teacher): data = S x 16 inputs then S targets (float32, 17 S values)."""
    if samples % 128 or not 128 <= samples <= 4096:
        raise ValueError("samples must be a multiple of 128 in [128, 4096]")
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((samples, N_IN)).astype(np.float32)
    teacher = pack(rng.normal(0.0, 1.0 / np.sqrt(N_IN), (N_IN, N_HIDDEN)),
                   rng.normal(0.0, 0.1, N_HIDDEN),
                   rng.normal(0.0, 1.0 / np.sqrt(N_HIDDEN), N_HIDDEN), 0.0)
    y = predict(teacher, X).astype(np.float32)
    return np.concatenate([X.reshape(-1), y]).astype(np.float32), teacher


def mlp_problem(data, bound: float = 1.0) -> OptimizationProblem:
    """OptimizationProblem of the MLP fit with box bounds [-bound, bound]^577."""
    return OptimizationProblem(mlp_regression, np.zeros(DIM, np.float32), None,
                               lb=np.full(DIM, -bound, np.float32), ub=np.full(DIM, bound, np.float32),
                               data=data)
