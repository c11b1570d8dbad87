"""Build recipe for libpps_cuda.so (sm_103a only).

Every ``.cu`` file in this directory is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -fmad=false`` and linked
into ``parallelparticleswarms.jl_gb300/lib/libpps_cuda.so``.  ``-fmad=false``
keeps nvcc from contracting ``a*b + c`` so every kernel performs exactly the
binary32 operations its source spells (fused multiply-adds are written as
``__fmaf_rn``).  The device headers that NVRTC compiles with a user
objective are embedded into the library as string literals
(``_build/pps_rtc_sources.inc``).  Run as ``python build.py [-v]``; the library is rebuilt only
when a source is newer than it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
PKG = HERE.parent
OUT_DIR = PKG / "lib"
OBJ_DIR = PKG / "_build"
LIB = OUT_DIR / "libpps_cuda.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-Xptxas", "-warn-spills",
    f"-I{INCLUDE}", f"-I{HERE}", f"-I{OBJ_DIR}",
]


# device headers that NVRTC compiles with the source of a user objective
# (pps_user.cu): embedded into the library as string literals
RTC_HEADERS = ["pps_device.cuh", "pps_state.cuh", "pps_publish.cuh", "pps_vec.cuh", "pps_objgrad.cuh", "pps_local.cuh",
               "pps_user_prelude.cuh", "pps_user_kernels.cuh"]
RTC_INC = OBJ_DIR / "pps_rtc_sources.inc"


def write_rtc_sources() -> None:
    """Write _build/pps_rtc_sources.inc: the NVRTC headers as raw string literals."""
    delim = "PPSRTC"
    lines = ["// generated by build.py from the headers below; do not edit", "namespace {"]
    names, texts = [], []
    for h in RTC_HEADERS:
        text = (HERE / h).read_text()
        if f"){delim}" in text:
            raise RuntimeError(f"{h} contains the raw-string delimiter")
        names.append(f'"{h}"')
        texts.append(f'R"{delim}({text}){delim}"')
    lines.append(f"constexpr int kRtcHeaderCount = {len(RTC_HEADERS)};")
    lines.append("const char* const kRtcHeaderNames[] = {" + ", ".join(names) + "};")
    lines.append("const char* const kRtcHeaderTexts[] = {\n" + ",\n".join(texts) + "};")
    lines.append("}  // namespace")
    body = "\n".join(lines) + "\n"
    if not RTC_INC.exists() or RTC_INC.read_text() != body:
        RTC_INC.write_text(body)


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpps_cuda.so")
    return cand


def sources() -> list[Path]:
    return sorted(HERE.glob("*.cu")) + sorted(HERE.glob("*.cpp"))


def headers() -> list[Path]:
    return sorted(HERE.glob("*.cuh")) + sorted(HERE.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _compile(src: Path, verbose: bool) -> Path:
    obj = OBJ_DIR / (src.name + ".o")
    cmd = [nvcc(), "-c", str(src), "-o", str(obj)] + NVCC_FLAGS
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        sys.stderr.write(r.stdout + r.stderr)
    return obj


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in sources() + headers() + [Path(__file__)])


def build(verbose: bool = False, force: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    write_rtc_sources()
    srcs = sources()
    workers = min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH + ["-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build(verbose=v, force="-f" in sys.argv or v))
