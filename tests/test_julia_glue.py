"""The Julia glue package (parallelparticleswarms.jl_gb300/julia/PPSCUDA), checked
without a Julia toolchain (none exists here): it ccalls every entry point
include/pps.h declares and nothing else, each one exported by libpps_cuda.so,
and the structs it passes by reference have pps.h's fields in pps.h's order
with matching types."""
import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
JL = ROOT / "parallelparticleswarms.jl_gb300" / "julia" / "PPSCUDA" / "src" / "PPSCUDA.jl"
HEADER = ROOT / "include" / "pps.h"

C_TO_JL = {"int32_t": "Int32", "int64_t": "Int64", "uint32_t": "UInt32", "uint64_t": "UInt64", "float": "Float32",
           "double": "Float64", "const float*": "Ptr{Float32}", "float*": "Ptr{Float32}"}


def _c_struct(name):
    text = HEADER.read_text()
    body = re.search(r"typedef struct " + name + r" \{(.*?)\} " + name + ";", text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(const float\*|float\*|int32_t|int64_t|uint32_t|uint64_t|float|double)\s+(\w+(?:\s*,\s*\w+)*)$",
                     decl)
        assert m, decl
        for name in m.group(2).split(","):  # one type, several declarators
            fields.append((name.strip(), C_TO_JL[m.group(1)]))
    return fields


def _jl_struct(name):
    text = JL.read_text()
    body = re.search(r"struct " + name + r"\n(.*?)\nend", text, re.S).group(1)
    return [tuple(x.strip() for x in line.split("::")) for line in body.strip().splitlines()]


def test_structs_match_the_header():
    assert _jl_struct("PPSProblem") == _c_struct("pps_problem")
    assert _jl_struct("PPSLocalOpts") == _c_struct("pps_local_opts")
    assert _jl_struct("PPSServeConfig") == _c_struct("pps_serve_config")
    assert _jl_struct("PPSServeStats") == _c_struct("pps_serve_stats")
    assert _jl_struct("PPSSwarmInfo") == _c_struct("pps_swarm_info")
    assert _jl_struct("PPSDeviceSwarm") == _c_struct("pps_device_swarm")


def test_every_ccall_is_declared_and_exported(pps):
    from parallelparticleswarms import _lib

    called = set(re.findall(r"ccall\(\(:(pps_\w+), lib\(\)\)", JL.read_text()))
    declared = set(re.findall(r"PPS_API\s+[\w\s\*]+?\b(pps_\w+)\s*\(", HEADER.read_text()))
    assert called <= declared, sorted(called - declared)
    assert declared <= called, ("entry points without a Julia binding", sorted(declared - called))
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    assert called <= set(re.findall(r"\bT\s+(pps_\w+)", out))


def test_package_layout():
    proj = (JL.parent.parent / "Project.toml").read_text()
    assert 'name = "PPSCUDA"' in proj and "ParallelParticleSwarms" in proj
    text = JL.read_text()
    assert text.count("module PPSCUDA") == 1 and text.rstrip().endswith("end # module")
