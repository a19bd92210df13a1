"""Builds libbfgpu.so (the engine, sm_103a) and, when asked, the CPU oracle.

Every translation unit is compiled by nvcc in parallel and linked into
code_mojo_gb300/_lib/libbfgpu.so with the CUDA runtime linked statically, so
the library needs nothing but the NVIDIA driver at run time.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
OBJDIR = PKG / "_build"
LIB = LIBDIR / "libbfgpu.so"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
SOURCES = ["api.cpp", "planner.cpp", "server.cpp", "gates.cu", "tile.cu", "perm.cu", "state_ops.cu", "measure.cu", "grover.cu", "batch.cu", "noalloc.cu", "blocks.cpp", "tblock.cu", "wire.cpp"]


def _deps_mtime() -> float:
    files = list(CSRC.glob("*")) + [ROOT / "include" / "bfgpu.h", Path(__file__)]
    return max(f.stat().st_mtime for f in files if f.is_file())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_engine(force: bool = False, verbose: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime >= _deps_mtime():
        return LIB
    OBJDIR.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    jobs = []
    for src in SOURCES:
        obj = OBJDIR / (src + ".o")
        cmd = [NVCC, *ARCH, *COMMON, "-I", str(ROOT / "include"), "-c", str(CSRC / src), "-o", str(obj)]
        if src.endswith(".cu"):
            cmd += ["-Xptxas", "-warn-spills"]
        jobs.append((cmd, obj))
    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(lambda j: _run(j[0]), jobs))
    tmp = LIB.with_suffix(".so.tmp")
    _run([NVCC, *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o in jobs], "-lpthread"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


def build_oracle(force: bool = False) -> Path:
    out = ROOT / "oracle" / "_build" / "liboracle.so"
    src = [ROOT / "oracle" / "oracle.cpp", ROOT / "oracle" / "oracle.h", ROOT / "include" / "bfgpu.h"]
    if out.exists() and not force and out.stat().st_mtime >= max(f.stat().st_mtime for f in src):
        return out
    _run(["make", "-s", "-C", str(ROOT / "oracle")])
    return out


if __name__ == "__main__":
    build_engine(force="--force" in sys.argv, verbose=True)
    build_oracle(force="--force" in sys.argv)
