"""The TMA-staged synchronous step against the register-prefetch step.

Every other parity test runs the library's default step kernel (k_sync_step,
the warps' own loads prefetched one dim pair ahead in registers) against the
oracle.  These run the cases of sync_kernel_cases.py once more in a child
process with PPS_SYNC_KERNEL=bulk (k_sync_step_bulk: the swarm state streamed
through a ring of shared-memory stages by bulk copies) and require the two
final states to be identical bit for bit: ragged last tiles, odd and single
dims, dims whose bounds take 12 kB and 48 kB of shared memory beside the
ring, many tiles per block, the graph-replayed run, and several ring shapes."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import sync_kernel_cases

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


def _child_states(tmp_path, **env_over):
    out = tmp_path / "child.npz"
    env = dict(os.environ)
    env.pop("PPS_SYNC_BULK", None)
    env.update(env_over)
    subprocess.run([sys.executable, str(HERE / "sync_kernel_cases.py"), str(out)], env=env, check=True,
                   timeout=900)
    return np.load(out)


@pytest.fixture(scope="module")
def default_states(pps):
    return sync_kernel_cases.run_cases(pps)


@pytest.mark.parametrize("shape", [None, "2,4", "8,2", "4,6"], ids=["default-ring", "2x4", "8x2", "4x6"])
def test_tma_step_equals_register_step(default_states, tmp_path, shape):
    """PPS_SYNC_BULK=dims,stages reshapes the ring (dims per stage, stages):
    neither the kernel nor the ring changes a bit."""
    env = {"PPS_SYNC_KERNEL": "bulk"}
    if shape:
        env["PPS_SYNC_BULK"] = shape
    other = _child_states(tmp_path, **env)
    assert set(default_states) == set(other.files)
    for k, v in default_states.items():
        assert np.array_equal(np.asarray(v), other[k], equal_nan=True), f"{k} differs (TMA-staged, ring {shape})"
