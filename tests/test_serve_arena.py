"""The serving arena's allocator on the CPU: tests/host/arena_check.cpp, built
by g++ against parallelparticleswarms.jl_gb300/csrc/pps_arena.h, drives random
allocation and release sequences and checks them against a plain model."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_arena_allocator(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "arena_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror",
                    "-I", str(ROOT / "parallelparticleswarms.jl_gb300" / "csrc"),
                    str(ROOT / "tests" / "host" / "arena_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "arena ok" in r.stdout
