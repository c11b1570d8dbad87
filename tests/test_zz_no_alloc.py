"""pps_sync_run_noalloc: the synchronous run on device buffers owned by the
caller, for callers that cannot let the library allocate (a pooled allocator
such as CUDA.jl's holds the memory, or a host framework hands out every
buffer).  Its output must equal pps_sync_run's on the same swarm, bit for bit
as every parity test here requires, on two calls in a row (the second call
continues the iteration counter and reuses the library's static scratch).

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _to_device(torch, a, ld):
    """(rows, n) float32 -> device tensor of shape (rows, ld), zero padding."""
    a = np.atleast_2d(np.asarray(a, np.float32))
    buf = np.zeros((a.shape[0], ld), np.float32)
    buf[:, : a.shape[1]] = a
    return torch.from_numpy(buf).cuda()


def test_noalloc_matches_sync_run_on_two_calls(pps):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    from parallelparticleswarms import _lib

    lib = _lib.load()
    D, n, K, seed = 24, 3000, 40, 17
    ld = (n + 31) // 32 * 32
    lb = np.full(D, -5.12, np.float32)
    ub = np.full(D, 5.12, np.float32)
    params = np.array([10.0], np.float32)
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(D, np.float32), params, lb=lb, ub=ub)
    with pps.Swarm(prob, n, seed=seed) as sw:
        sw.init()
        st = sw.state()
        x, v, pb = (_to_device(torch, st[k], ld) for k in ("x", "v", "pbest"))
        pc, cc = (_to_device(torch, st[k], ld) for k in ("pcost", "cost"))
        dlb, dub = _to_device(torch, lb, D), _to_device(torch, ub, D)
        g = torch.zeros(D, dtype=torch.float32, device="cuda")
        ds = _lib.DeviceSwarm(n, ld, D, x.data_ptr(), v.data_ptr(), pb.data_ptr(), pc.data_ptr(), cc.data_ptr(),
                              dlb.data_ptr(), dub.data_ptr(), g.data_ptr())
        for call in range(2):
            gcost, gidx = ctypes.c_float(), ctypes.c_int64()
            torch.cuda.synchronize()
            rc = lib.pps_sync_run_noalloc(2, _lib.fptr(params), 1, ctypes.byref(ds), seed, call * K, K, 0.7298, 1.0,
                                          1.4962, 1.4962, 0, None, ctypes.byref(gcost), ctypes.byref(gidx))
            assert rc == 0, lib.pps_last_error()
            torch.cuda.synchronize()
            sw.sync_run(K)
            want = sw.state()
            u, wcost, widx = sw.gbest()
            for name, t in (("x", x), ("v", v), ("pbest", pb)):
                got = t.cpu().numpy()[:, :n]
                assert np.array_equal(got, want[name]), f"call {call + 1}: {name} differs"
            assert np.array_equal(pc.cpu().numpy()[0, :n], want["pcost"]), f"call {call + 1}: pcost differs"
            assert np.array_equal(cc.cpu().numpy()[0, :n], want["cost"]), f"call {call + 1}: cost differs"
            assert np.array_equal(g.cpu().numpy(), u), f"call {call + 1}: global best differs"
            assert gidx.value == widx and np.float32(gcost.value) == np.float32(wcost)


def test_noalloc_rejects_oversize_requests(pps):
    from parallelparticleswarms import _lib

    lib = _lib.load()
    big = (1 << 20) + 32
    ds = _lib.DeviceSwarm(big, big, 4, 16, 16, 16, 16, 16, 16, 16, 16)
    rc = lib.pps_sync_run_noalloc(2, None, 0, ctypes.byref(ds), 0, 0, 1, 0.7, 1.0, 1.4, 1.4, 0, None, None, None)
    assert rc == _lib.EINVAL
    assert b"1048576" in lib.pps_last_error()
