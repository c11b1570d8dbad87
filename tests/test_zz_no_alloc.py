"""pps_sync_run_noalloc: the synchronous run on device buffers owned by the
caller, for callers that cannot let the library allocate (a pooled allocator
such as CUDA.jl's holds the memory, or a host framework hands out every
buffer).  Its output must equal pps_sync_run's on the same swarm, bit for bit
as every parity test here requires, on two calls in a row (the second call
continues the iteration counter and reuses the library's static scratch),
with either global-best rule and on the legacy default stream as well as on
a stream of the caller's.  The second call must not change the device's free
memory: the entry point exists because it allocates nothing.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest


def _to_device(torch, a, ld):
    """(rows, n) float32 -> device tensor of shape (rows, ld), zero padding."""
    a = np.atleast_2d(np.asarray(a, np.float32))
    buf = np.zeros((a.shape[0], ld), np.float32)
    buf[:, : a.shape[1]] = a
    return torch.from_numpy(buf).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("from_position", [False, True], ids=["gbest_from_pbest", "gbest_from_position"])
@pytest.mark.parametrize("own_stream", [False, True], ids=["default_stream", "caller_stream"])
@pytest.mark.parametrize("n", [3000, 990], ids=["n3000", "n990-ld992"])
def test_noalloc_matches_sync_run_on_two_calls(pps, from_position, own_stream, n):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    from parallelparticleswarms import _lib

    lib = _lib.load()
    D, K, seed = 24, 40, 17  # ld = 992 for n = 990: a last tile of 32 particles (half a warp's)
    ld = (n + 31) // 32 * 32
    lb = np.full(D, -5.12, np.float32)
    ub = np.full(D, 5.12, np.float32)
    params = np.array([10.0], np.float32)
    flags = _lib.FLAG_GBEST_FROM_POSITION if from_position else 0
    stream = torch.cuda.Stream() if own_stream else None
    handle = ctypes.c_void_p(stream.cuda_stream) if own_stream else None
    prob = pps.OptimizationProblem(pps.rastrigin, np.zeros(D, np.float32), params, lb=lb, ub=ub)
    with pps.Swarm(prob, n, seed=seed, gbest_from_position=from_position) as sw:
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
            free_before = torch.cuda.mem_get_info()[0]
            rc = lib.pps_sync_run_noalloc(2, _lib.fptr(params), 1, ctypes.byref(ds), seed, call * K, K, 0.7298, 1.0,
                                          1.4962, 1.4962, flags, handle, ctypes.byref(gcost), ctypes.byref(gidx))
            assert rc == 0, lib.pps_last_error()
            torch.cuda.synchronize()
            if call == 1:  # the first call on a device may load the library's device code
                assert torch.cuda.mem_get_info()[0] == free_before, "the call changed the device's free memory"
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
    """Checked on the host, before any device work (no GPU needed)."""
    from parallelparticleswarms import _lib

    lib = _lib.load()
    big = (1 << 20) + 32
    ds = _lib.DeviceSwarm(big, big, 4, 16, 16, 16, 16, 16, 16, 16, 16)
    rc = lib.pps_sync_run_noalloc(2, None, 0, ctypes.byref(ds), 0, 0, 1, 0.7, 1.0, 1.4, 1.4, 0, None, None, None)
    assert rc == _lib.EINVAL
    assert b"1048576" in lib.pps_last_error()


def test_noalloc_rejects_bad_coefficients_and_counter_overflow(pps):
    """Non-finite coefficients and an iteration counter that would wrap (the
    Philox draws of an iteration depend on its number) fail before any device
    work, as they do for pps_sync_run."""
    from parallelparticleswarms import _lib

    lib = _lib.load()
    ds = _lib.DeviceSwarm(64, 64, 4, 16, 16, 16, 16, 16, 16, 16, 16)
    nan = float("nan")
    for w, wdamp, c1, c2 in ((nan, 1.0, 1.4, 1.4), (0.7, float("inf"), 1.4, 1.4), (0.7, 1.0, nan, 1.4),
                             (0.7, 1.0, 1.4, -float("inf"))):
        rc = lib.pps_sync_run_noalloc(2, None, 0, ctypes.byref(ds), 0, 0, 1, w, wdamp, c1, c2, 0, None, None, None)
        assert rc == _lib.EINVAL and b"finite" in lib.pps_last_error()
    rc = lib.pps_sync_run_noalloc(2, None, 0, ctypes.byref(ds), 0, 0xFFFFFFF0, 32, 0.7, 1.0, 1.4, 1.4, 0, None,
                                  None, None)
    assert rc == _lib.EINVAL and b"overflow" in lib.pps_last_error()
