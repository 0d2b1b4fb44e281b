"""Build recipe for the GB300 position-based-fluids library.

Compiles every CUDA translation unit for sm_103a (one -gencode, no PTX
fallback) and the host C++ units, in parallel, and links them in-tree into
``position-based-fluids_gb300/libpbf_gb300.so`` plus the headless runner
``position-based-fluids_gb300/pbf_run``.  Objects go to ``_build/`` beside
this file.  No cmake, no torch extension machinery: plain nvcc / g++.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
SRC = PKG_DIR / "csrc"
OBJ = PKG_DIR / "_build"
REPO = PKG_DIR.parent
LIB = PKG_DIR / "libpbf_gb300.so"
RUNNER = PKG_DIR / "pbf_run"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc") if (CUDA_HOME / "bin" / "nvcc").exists() else "nvcc"
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC_FLAGS = [*ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I", str(REPO / "include")]
# Translation units whose arithmetic must not be contracted into FMAs.
NO_FMAD = {"pbf_refcompat.cu", "pbf_render.cu"}
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
             "-Wno-unused-parameter", "-I", str(CUDA_HOME / "include"), "-I", str(REPO / "include")]

CU_SOURCES = ["pbf_sort.cu", "pbf_paper.cu", "pbf_tile.cu", "pbf_refcompat.cu", "pbf_noalloc.cu",
              "pbf_render.cu"]
CPP_SOURCES = ["pbf_params.cpp", "pbf_scenario.cpp", "pbf_sim.cpp", "pbf_batch.cpp", "pbf_server.cpp",
               "Simulation.cpp"]
RUNNER_SOURCES = ["pbf_run.cpp"]
HEADERS = ["pbf_internal.cuh", "pbf_device.cuh", "pbf_paper.cuh", "pbf_host.hpp", "Simulation.hpp"]


def _run(cmd: list[str]) -> str:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    return proc.stdout + proc.stderr


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _compile_jobs(force: bool, extra_nvcc: list[str]) -> tuple[list[list[str]], list[Path]]:
    OBJ.mkdir(exist_ok=True)
    common_deps = [SRC / h for h in HEADERS] + [REPO / "include" / "pbf.h"]
    jobs, objs = [], []
    for name in CU_SOURCES:
        src = SRC / name
        obj = OBJ / (name + ".o")
        objs.append(obj)
        flags = NVCC_FLAGS + (["-fmad=false", "-Xcompiler", "-ffp-contract=off"]
                              if name in NO_FMAD else []) + extra_nvcc
        if force or _stale(obj, [src, *common_deps]):
            jobs.append([NVCC, *flags, "-c", str(src), "-o", str(obj)])
    for name in CPP_SOURCES:
        src = SRC / name
        obj = OBJ / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *common_deps]):
            jobs.append([CXX, *CXX_FLAGS, "-c", str(src), "-o", str(obj)])
    return jobs, objs


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    """Builds libpbf_gb300.so and pbf_run; returns the library path."""
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    jobs, objs = _compile_jobs(force or verbose_ptxas, extra)
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "--cudart", "static", "-o", str(LIB), *map(str, objs)])
    runner_src = [SRC / s for s in RUNNER_SOURCES]
    if force or _stale(RUNNER, runner_src + [LIB]):
        _run([CXX, *CXX_FLAGS, *map(str, runner_src), "-o", str(RUNNER),
              f"-L{PKG_DIR}", "-lpbf_gb300", f"-Wl,-rpath,{PKG_DIR}"])
    if verbose_ptxas:
        for log in logs:
            sys.stdout.write(log)
    return LIB


def clean() -> None:
    if OBJ.exists():
        shutil.rmtree(OBJ)
    for p in (LIB, RUNNER):
        if p.exists():
            p.unlink()


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
