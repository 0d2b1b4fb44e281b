"""Build recipe for the oracle (TEST INFRASTRUCTURE, never part of the product).

Two libraries come out of it:

* ``oracle/_build/libpbforacle.so`` -- the CPU restatement
  (``oracle/pbf_oracle.cpp``), built from this repository's own sources.
* ``oracle/_ref/libpbfref.so`` -- the reference's own live kernels
  (MrMagne/position-based-fluids ``src/kernels/*.cl``) compiled as C++ through
  ``oracle/clshim.hpp`` and launched by ``oracle/ref_launch.cpp``.

The reference sources are read where they lie: the checkout named by the
environment variable ``PBF_REFERENCE_ROOT`` (default ``/root/reference``);
they are never copied into the repository.  The first stage runs the C++
preprocessor over each ``.cl`` file alone (comments dropped, the
``USE_LINKEDCELL`` branches of the active build resolved, no header expanded)
and writes the kernel text to ``oracle/_ref/<kernel>.pre.cl``; the second
compiles those units as C++ with the shim force-included, so the system
headers come from the host that compiles them.  ``oracle/_ref`` is
git-ignored.  Where the reference tree is absent (the GPU host) the second
stage still runs from any ``.pre.cl`` files present, so the compiled reference
can be rebuilt for that host's architecture; without them the oracle
restatement is the only CPU implementation.

All oracle code is built with ``-ffp-contract=off`` and without fast-math, so
x86-64 and aarch64 builds give bit-identical results.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
REF_DIR = ORACLE_DIR / "_ref"
# The reference checkout: PBF_REFERENCE_ROOT, by default /root/reference.
REFERENCE_ROOT = Path(os.environ.get("PBF_REFERENCE_ROOT", "/root/reference"))
REFERENCE_KERNELS = REFERENCE_ROOT / "src" / "kernels"
REFERENCE_SCENARIOS = REFERENCE_ROOT / "assets" / "scenarios"

# The kernels of the reference's active (linked-cell) build, src/main.cpp:67-84.
LIVE_KERNELS = [
    "predict_positions",
    "init_cells_old",
    "update_cells",
    "compute_scaling",
    "compute_delta",
    "update_predicted",
    "update_velocities",
    "apply_vorticity_and_viscosity",
    "update_positions",
]

CXX = os.environ.get("CXX", "g++")
COMMON = ["-std=gnu++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp"]

RESTATEMENT_LIB = BUILD_DIR / "libpbforacle.so"
REFERENCE_LIB = REF_DIR / "libpbfref.so"


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources if s.exists())


def build_restatement(force: bool = False) -> Path:
    BUILD_DIR.mkdir(exist_ok=True)
    srcs = [ORACLE_DIR / "pbf_oracle.cpp", ORACLE_DIR / "pbf_oracle.h"]
    if force or _stale(RESTATEMENT_LIB, srcs):
        _run([CXX, *COMMON, "-shared", str(srcs[0]), "-o", str(RESTATEMENT_LIB)])
    return RESTATEMENT_LIB


def _shim_for(kernel: str) -> Path:
    return ORACLE_DIR / ("clshim_predict.hpp" if kernel == "predict_positions" else "clshim.hpp")


def preprocess_reference() -> bool:
    """Stage 1: needs the reference tree; writes oracle/_ref/<kernel>.pre.cl."""
    if not REFERENCE_KERNELS.is_dir():
        return False
    REF_DIR.mkdir(exist_ok=True)
    jobs = []
    for k in LIVE_KERNELS:
        src = REFERENCE_KERNELS / f"{k}.cl"
        out = REF_DIR / f"{k}.pre.cl"
        if _stale(out, [src]):
            jobs.append([CXX, "-E", "-P", "-DUSE_LINKEDCELL", "-x", "c", str(src), "-o", str(out)])
    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(_run, jobs))
    return True


def build_reference(force: bool = False) -> Path | None:
    """Stage 1 (if the reference tree is here) then stage 2."""
    preprocess_reference()
    units = [REF_DIR / f"{k}.pre.cl" for k in LIVE_KERNELS]
    if not all(u.exists() for u in units):
        return None
    launcher = ORACLE_DIR / "ref_launch.cpp"
    deps = units + [launcher, ORACLE_DIR / "clshim.hpp", ORACLE_DIR / "clshim_predict.hpp"]
    if not (force or _stale(REFERENCE_LIB, deps)):
        return REFERENCE_LIB
    objs = []
    jobs = []
    for k, u in zip(LIVE_KERNELS, units):
        o = REF_DIR / f"{k}.o"
        objs.append(o)
        jobs.append([CXX, *COMMON, "-w", "-x", "c++", "-include", str(_shim_for(k)), "-c", str(u), "-o", str(o)])
    dobj = REF_DIR / "ref_launch.o"
    jobs.append([CXX, *COMMON, "-c", str(launcher), "-o", str(dobj)])
    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(_run, jobs))
    _run([CXX, *COMMON, "-shared", *map(str, objs), str(dobj), "-o", str(REFERENCE_LIB)])
    return REFERENCE_LIB


def build(force: bool = False) -> dict:
    out = {"restatement": str(build_restatement(force))}
    ref = build_reference(force)
    out["reference"] = str(ref) if ref else None
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
