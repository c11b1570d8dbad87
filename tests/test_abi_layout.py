"""The Python ctypes mirrors of the C ABI's structs (parallelparticleswarms/_lib.py)
have the layout include/pps.h gives them: a C program compiled against the
header prints every field's offset and each struct's size, and ctypes must
agree field by field (a renamed, reordered or resized field fails here, not
as a silently misread argument on the GPU)."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import pytest

from parallelparticleswarms import _lib

ROOT = Path(__file__).resolve().parents[1]

STRUCTS = {
    "pps_problem": _lib.Problem,
    "pps_swarm_info": _lib.SwarmInfo,
    "pps_local_opts": _lib.LocalOpts,
    "pps_serve_config": _lib.ServeConfig,
    "pps_serve_stats": _lib.ServeStats,
    "pps_device_swarm": _lib.DeviceSwarm,
}


def _c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "pps.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        struct, field, value = line.split()
        table[(struct, field)] = int(value)
    return table


def test_ctypes_structs_match_the_header(tmp_path):
    table = _c_layout(tmp_path)
    for cname, py in STRUCTS.items():
        assert ctypes.sizeof(py) == table[(cname, "sizeof")], cname
        for fname, _ in py._fields_:
            assert getattr(py, fname).offset == table[(cname, fname)], (cname, fname)
