"""The MLP-regression objective's CPU restatement (examples/neural_network/nn.jl:
a network's loss as a PSO objective), pinned against an independent numpy
restatement, plus host-side checks of the problem builder and of the C ABI's
argument validation (no GPU needed)."""
import ctypes

import numpy as np
import pytest


def _bf16_numpy(a):
    """Round float32 to bfloat16 (nearest, ties to even) with integer arithmetic."""
    b = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def _loss_numpy(x, X, y):
    W1 = _bf16_numpy(x[:512]).astype(np.float64).reshape(16, 32)
    h = _bf16_numpy(X).astype(np.float64) @ W1 + x[512:544].astype(np.float64)
    o = np.tanh(h) @ x[544:576].astype(np.float64) + np.float64(x[576])
    return float(np.mean((o - y.astype(np.float64)) ** 2))


def test_bf16_round_known_answers(orc):
    lib = orc.load()
    cases = {
        1.0: 1.0,
        1.00390625: 1.0,          # 1 + 2^-8: a tie, rounds to the even neighbour 1.0
        1.01171875: 1.015625,     # 1 + 3 * 2^-8: a tie, rounds up to even
        1.0078125: 1.0078125,     # exactly representable
        3.14159: 3.140625,
        -2.5: -2.5,
        65504.0: 65536.0,
    }
    for v, want in cases.items():
        assert lib.orc_bf16_round(v) == want, v
    assert np.isinf(lib.orc_bf16_round(np.inf))
    assert np.isnan(lib.orc_bf16_round(np.nan))


def test_bf16_round_matches_numpy(orc):
    lib = orc.load()
    rng = np.random.default_rng(3)
    vals = np.concatenate([rng.standard_normal(4000), rng.uniform(-1e6, 1e6, 1000),
                           rng.uniform(-1e-30, 1e-30, 1000)]).astype(np.float32)
    want = _bf16_numpy(vals)
    got = np.array([lib.orc_bf16_round(float(v)) for v in vals], np.float32)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("samples", [128, 1024])
def test_mlp_loss_matches_numpy(orc, samples):
    import parallelparticleswarms as pps

    data, teacher = pps.mlp.teacher_task(samples, seed=5)
    X = data[:samples * 16].reshape(samples, 16)
    y = data[samples * 16:]
    rng = np.random.default_rng(1)
    for k in range(6):
        x = rng.uniform(-1, 1, 577).astype(np.float32)
        assert orc.mlp_loss(x, X, y) == pytest.approx(_loss_numpy(x, X, y), rel=1e-12)
    # the teacher fits its own data up to the bfloat16 rounding of the GEMM operands
    assert orc.mlp_loss(teacher, X, y) < 1e-3 * float(np.var(y))


def test_teacher_task_layout():
    import parallelparticleswarms as pps

    data, teacher = pps.mlp.teacher_task(256, seed=2)
    assert data.dtype == np.float32 and data.size == 17 * 256
    X = data[:256 * 16].reshape(256, 16)
    np.testing.assert_allclose(data[256 * 16:], pps.mlp.predict(teacher, X), rtol=1e-6, atol=1e-6)
    W1, b1, w2, b2 = pps.mlp.unpack(teacher)
    assert np.array_equal(pps.mlp.pack(W1, b1, w2, b2), teacher)
    with pytest.raises(ValueError):
        pps.mlp.teacher_task(100)


def test_oracle_pso_reduces_mlp_loss(orc):
    import parallelparticleswarms as pps

    data, _ = pps.mlp.teacher_task(128, seed=9)
    prob = pps.mlp.mlp_problem(data)
    op = orc.OracleProblem(6, 577, prob.lb, prob.ub, mlp_data=data)
    sw = orc.OracleSwarm(op, 256, 4).init()
    first = sw.gcost
    sw.sync_run(30)
    assert sw.gcost < 0.7 * first


def test_c_abi_rejects_bad_mlp_problems(pps):
    """Argument checks run before any CUDA call."""
    from parallelparticleswarms import _lib

    lib = _lib.load()
    data, _ = pps.mlp.teacher_task(128)
    good = pps.mlp.mlp_problem(data)
    bad = [
        good.remake(u0=np.zeros(576, np.float32), lb=None, ub=None),   # wrong dim
        good.remake(data=data[:-1]),                                    # not 17 S floats
        good.remake(data=np.zeros(17 * 100, np.float32)),               # S not a multiple of 128
        good.remake(data=np.zeros(17 * 4224, np.float32)),              # S above 4096
    ]
    x = np.zeros(577, np.float32)
    f = np.zeros(1, np.float32)
    for p in bad:
        pr = p.to_c()
        assert lib.pps_eval_objective(ctypes.byref(pr), 1, _lib.fptr(x), _lib.fptr(f)) == _lib.EINVAL
