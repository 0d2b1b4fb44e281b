"""CPU oracle for the position-based-fluids step -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this package, and only as the oracle results are compared
against (or the timed CPU baseline).  The product library never links or calls it.

Two native libraries back it (``oracle/build.py`` builds both):

* ``restatement`` -- ``oracle/pbf_oracle.cpp``: the reference's live kernels
  restated (REF_COMPAT, float and double), the PBF_PAPER equations in double,
  and the sort-path intent (hash, stable sort, inclusive cell ranges);
* ``reference`` -- the reference's own ``src/kernels/*.cl`` compiled as C++
  (``oracle/ref_launch.cpp``); present only where the reference tree, or its
  preprocessed kernel text in ``oracle/_ref``, was available at build time.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import build as _build

_F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_F64P = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_U32P = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class Config(C.Structure):
    """The .par values the reference's simulation reads (src/Parameters.hpp)."""

    _fields_ = [
        ("x_min", C.c_float), ("x_max", C.c_float),
        ("y_min", C.c_float), ("y_max", C.c_float),
        ("z_min", C.c_float), ("z_max", C.c_float),
        ("x_n", C.c_float), ("y_n", C.c_float), ("z_n", C.c_float),
        ("timestep_length", C.c_float), ("rest_density", C.c_float),
    ]

    @property
    def ncells(self) -> int:
        return int(self.x_n) * int(self.y_n) * int(self.z_n)


class PaperParams(C.Structure):
    _fields_ = [
        ("box_min", C.c_double * 3), ("box_max", C.c_double * 3),
        ("n_cells", C.c_int32 * 3), ("iterations", C.c_int32),
        ("dt", C.c_double), ("rest_density", C.c_double), ("h", C.c_double),
        ("relax_eps", C.c_double), ("scorr_k", C.c_double), ("scorr_dq", C.c_double),
        ("xsph_c", C.c_double), ("vort_eps", C.c_double), ("gravity_y", C.c_double),
        ("wall_margin", C.c_double), ("scorr_n", C.c_int32), ("pad_", C.c_int32),
    ]


_lib_restatement = None
_lib_reference = None
_ref_checked = False


def restatement():
    global _lib_restatement
    if _lib_restatement is None:
        path = _build.build_restatement()
        lib = C.CDLL(str(path))
        cfgp = C.POINTER(Config)
        lib.oracle_ref_constants.argtypes = [cfgp, _F32P]
        lib.oracle_cell_hash.argtypes = [cfgp, _F32P, C.c_uint32, _U32P]
        lib.oracle_sort_cells.argtypes = [_U32P, C.c_uint32, _U32P, _U32P]
        lib.oracle_find_cells.argtypes = [_U32P, C.c_uint32, C.c_uint32, _I32P]
        lib.oracle_refcompat_steps_f32.argtypes = [
            cfgp, C.c_uint32, _F32P, _F32P, C.c_uint32, C.c_float, C.c_int, C.c_void_p, C.c_void_p]
        lib.oracle_refcompat_steps_f64.argtypes = [
            cfgp, C.c_uint32, _F64P, _F64P, C.c_uint32, C.c_double, C.c_int]
        for fn in (lib.oracle_paper_steps_f64, lib.oracle_paper_steps_f32):
            fn.argtypes = [C.POINTER(PaperParams), C.c_uint32, _F64P, _F64P, C.c_uint32, C.c_double,
                           C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib_restatement = lib
    return _lib_restatement


def reference():
    """The compiled reference kernels, or None where they cannot be built."""
    global _lib_reference, _ref_checked
    if not _ref_checked:
        _ref_checked = True
        path = _build.build_reference()
        if path is not None:
            lib = C.CDLL(str(path))
            cfgp = C.POINTER(Config)
            lib.ref_constants.argtypes = [cfgp, _F32P]
            lib.ref_run_steps.argtypes = [
                cfgp, C.c_uint32, _F32P, _F32P, C.c_uint32, C.c_float, C.c_int, C.c_int,
                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
            lib.ref_build_cells.argtypes = [cfgp, C.c_uint32, _F32P, _I32P, _I32P]
            lib.ref_compute_scaling.argtypes = [cfgp, C.c_uint32, _F32P, _I32P, _I32P, _F32P]
            _lib_reference = lib
    return _lib_reference


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"oracle call {what} failed with status {rc}")


# ---------------------------------------------------------------- restatement
def ref_constants(cfg: Config) -> np.ndarray:
    out = np.zeros(18, np.float32)
    _check(restatement().oracle_ref_constants(C.byref(cfg), out), "ref_constants")
    return out


def cell_hash(cfg: Config, pred4: np.ndarray) -> np.ndarray:
    pred4 = np.ascontiguousarray(pred4, np.float32)
    n = pred4.shape[0]
    out = np.zeros(n, np.uint32)
    _check(restatement().oracle_cell_hash(C.byref(cfg), pred4.reshape(-1), n, out), "cell_hash")
    return out


def sort_cells(hash_: np.ndarray):
    hash_ = np.ascontiguousarray(hash_, np.uint32)
    n = hash_.shape[0]
    sk = np.zeros(n, np.uint32)
    perm = np.zeros(n, np.uint32)
    _check(restatement().oracle_sort_cells(hash_, n, sk, perm), "sort_cells")
    return sk, perm


def find_cells(sorted_hash: np.ndarray, ncells: int) -> np.ndarray:
    sorted_hash = np.ascontiguousarray(sorted_hash, np.uint32)
    out = np.zeros(2 * ncells, np.int32)
    _check(restatement().oracle_find_cells(sorted_hash, sorted_hash.shape[0], ncells, out), "find_cells")
    return out.reshape(ncells, 2)


def refcompat_steps_f32(cfg: Config, pos4, vel4, steps: int, wave: float = 0.0, threads: int = 0,
                        want_predicted: bool = False, want_scaling: bool = False):
    pos = np.array(pos4, np.float32, copy=True).reshape(-1, 4)
    vel = np.array(vel4, np.float32, copy=True).reshape(-1, 4)
    n = pos.shape[0]
    pred = np.zeros((n, 4), np.float32) if want_predicted else None
    sc = np.zeros(n, np.float32) if want_scaling else None
    _check(restatement().oracle_refcompat_steps_f32(
        C.byref(cfg), n, pos.reshape(-1), vel.reshape(-1), steps, wave, threads, _ptr(pred), _ptr(sc)),
        "refcompat_steps_f32")
    return pos, vel, pred, sc


def refcompat_steps_f64(cfg: Config, pos4, vel4, steps: int, wave: float = 0.0, threads: int = 0):
    pos = np.array(pos4, np.float64, copy=True).reshape(-1, 4)
    vel = np.array(vel4, np.float64, copy=True).reshape(-1, 4)
    n = pos.shape[0]
    _check(restatement().oracle_refcompat_steps_f64(
        C.byref(cfg), n, pos.reshape(-1), vel.reshape(-1), steps, wave, threads), "refcompat_steps_f64")
    return pos, vel


def paper_steps_f64(prm: PaperParams, pos4, vel4, steps: int, wave: float = 0.0, threads: int = 0,
                    precision: str = "f64"):
    """Returns (pos4, vel4, density, lambda, neighbour_count) after `steps`.
    precision="f32" evaluates the same algorithm in binary32."""
    pos = np.array(pos4, np.float64, copy=True).reshape(-1, 4)
    vel = np.array(vel4, np.float64, copy=True).reshape(-1, 4)
    n = pos.shape[0]
    dens = np.zeros(n, np.float64)
    lam = np.zeros(n, np.float64)
    cnt = np.zeros(n, np.uint32)
    fn = restatement().oracle_paper_steps_f64 if precision == "f64" else restatement().oracle_paper_steps_f32
    _check(fn(C.byref(prm), n, pos.reshape(-1), vel.reshape(-1), steps, wave, threads,
              _ptr(dens), _ptr(lam), _ptr(cnt)), "paper_steps")
    return pos, vel, dens, lam, cnt


# ----------------------------------------------------------- synthetic scenes
# The benchmark scenes built on the oracle side, so that a CPU run of the
# reference's kernels needs nothing from the product library.  The lattice
# and jitter follow the product's seeded block generator (lattice order of
# the reference's tools/gen_grid.py:1-49, x outermost and z innermost; three
# splitmix64 draws per particle, x then y then z); tests check the two
# bit for bit.
_SPLITMIX_GAMMA = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, count: int) -> np.ndarray:
    """The first `count` outputs of Vigna's splitmix64 generator from state
    `seed` (state += gamma, then the two xor-shift-multiply rounds)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed & (2**64 - 1)) + _SPLITMIX_GAMMA * np.arange(1, count + 1, dtype=np.uint64)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def generate_block(origin, dims, spacing: float, jitter: float, mass: float, seed: int):
    """(pos4, vel4) in the dumpData layout of a jittered lattice at rest:
    x = origin + index * spacing + (2u - 1) * jitter per coordinate, u the
    top 53 bits of a splitmix64 draw, evaluated in double and rounded once
    to binary32 (origin, spacing and jitter are binary32 values)."""
    nx, ny, nz = (int(d) for d in dims)
    n = nx * ny * nz
    idx = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"),
                   axis=-1).reshape(n, 3).astype(np.float64)
    u = (splitmix64(seed, 3 * n) >> np.uint64(11)).astype(np.float64).reshape(n, 3) * (1.0 / 9007199254740992.0)
    off = (2.0 * u - 1.0) * float(np.float32(jitter))
    o = np.asarray(origin, np.float32).astype(np.float64)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = (o + idx * float(np.float32(spacing)) + off).astype(np.float32)
    vel = np.zeros((n, 4), np.float32)
    vel[:, 3] = np.float32(mass)
    return pos, vel


def dam_break_scene(dims, box, seed: int = 0x5EED):
    """A benchmark dam break in the reference's units: a block at spacing
    0.05 (h = 0.1) in the box's minimum corner, h/4 from each wall, jitter
    0.01 spacing, mass 1000 * 0.05^3, cells of size h, dt = 1/120 and
    number density 1/0.05^3.  Returns (Config, pos4, vel4)."""
    h, spacing = 0.1, 0.05
    cells = [int(round(b / h)) for b in box]
    cfg = Config(0.0, box[0], 0.0, box[1], 0.0, box[2], cells[0], cells[1], cells[2],
                 1.0 / 120.0, 1.0 / spacing ** 3)
    m = 0.25 * h
    pos, vel = generate_block((m, m, m), dims, spacing, 0.01 * spacing, 1000.0 * spacing ** 3, seed)
    return cfg, pos, vel


def scene_small(seed: int = 0x5EED):
    """The 32,768-particle dam break (32^3 block in a 1.6 x 1.6 x 3.2 box,
    16 x 16 x 32 cells)."""
    return dam_break_scene((32, 32, 32), (1.6, 1.6, 3.2), seed)


def benchmark_paper_params(cfg: "Config") -> PaperParams:
    """The FP64 oracle's parameters of the benchmark's paper equations on
    `cfg`'s box: h 0.1, 4 iterations, relaxation 600, s_corr k 0.1 n 4
    dq 0.2 h, XSPH 0.01, vorticity 0.0005, gravity -9.81 along y, walls h/4
    inside the box; each value rounded to binary32 first, as the library's
    parameter block holds it."""
    f = lambda v: float(np.float32(v))  # noqa: E731
    o = PaperParams()
    o.box_min[:] = [cfg.x_min, cfg.y_min, cfg.z_min]
    o.box_max[:] = [cfg.x_max, cfg.y_max, cfg.z_max]
    o.n_cells[:] = [int(cfg.x_n), int(cfg.y_n), int(cfg.z_n)]
    o.iterations = 4
    o.dt = cfg.timestep_length
    o.rest_density = cfg.rest_density
    o.h = f(0.1)
    o.relax_eps = f(600.0)
    o.scorr_k = f(0.1)
    o.scorr_dq = f(0.2)
    o.scorr_n = 4
    o.xsph_c = f(0.01)
    o.vort_eps = f(0.0005)
    o.gravity_y = f(-9.81)
    o.wall_margin = f(0.25 * f(0.1))
    return o


def scene_1m(seed: int = 0x5EED):
    """The 1,048,576-particle headline scene (128 x 128 x 64 block, 6.4 m
    cube, 64^3 cells)."""
    return dam_break_scene((128, 128, 64), (6.4, 6.4, 6.4), seed)


def scene_4m(seed: int = 0x5EED):
    """The 4,194,304-particle double dam break: two 128^3 blocks on the floor
    at opposite x ends of a 12.8 x 12.8 x 6.4 box (128 x 128 x 64 cells), the
    second block seeded with seed + 1."""
    cfg, a_pos, a_vel = dam_break_scene((128, 128, 128), (12.8, 12.8, 6.4), seed)
    m = 0.025
    bx = 12.8 - m - 127 * 0.05
    b_pos, b_vel = generate_block((bx, m, m), (128, 128, 128), 0.05, 0.01 * 0.05, 1000.0 * 0.05 ** 3,
                                  seed + 1)
    return cfg, np.concatenate([a_pos, b_pos]), np.concatenate([a_vel, b_vel])


# ------------------------------------------------------------ compiled reference
def reference_available() -> bool:
    return reference() is not None


def reference_constants(cfg: Config) -> np.ndarray:
    out = np.zeros(18, np.float32)
    _check(reference().ref_constants(C.byref(cfg), out), "ref_constants")
    return out


def reference_steps(cfg: Config, pos4, vel4, steps: int, wave: float = 0.0, threads: int = 0,
                    parallel_cells: bool = False):
    """Runs the reference's own kernels; returns (pos4, vel4, predicted4,
    scaling, cells, list) from the last step."""
    pos = np.array(pos4, np.float32, copy=True).reshape(-1, 4)
    vel = np.array(vel4, np.float32, copy=True).reshape(-1, 4)
    n = pos.shape[0]
    pred = np.zeros((n, 4), np.float32)
    sc = np.zeros(n, np.float32)
    cells = np.zeros(cfg.ncells, np.int32)
    lst = np.zeros(n, np.int32)
    _check(reference().ref_run_steps(
        C.byref(cfg), n, pos.reshape(-1), vel.reshape(-1), steps, wave, threads, int(parallel_cells),
        _ptr(pred), _ptr(sc), _ptr(cells), _ptr(lst)), "ref_run_steps")
    return pos, vel, pred, sc, cells, lst


def reference_build_cells(cfg: Config, pred4):
    pred = np.ascontiguousarray(pred4, np.float32).reshape(-1, 4)
    n = pred.shape[0]
    cells = np.zeros(cfg.ncells, np.int32)
    lst = np.zeros(n, np.int32)
    _check(reference().ref_build_cells(C.byref(cfg), n, pred.reshape(-1), cells, lst), "ref_build_cells")
    return cells, lst


def cells_from_lists(cells: np.ndarray, lst: np.ndarray) -> dict[int, list[int]]:
    """Walks the reference's linked cell lists: cell -> particle indices, in
    list order."""
    out: dict[int, list[int]] = {}
    for c in np.nonzero(cells >= 0)[0]:
        j = int(cells[c])
        members = []
        guard = 0
        while j != -1:
            members.append(j)
            j = int(lst[j])
            guard += 1
            if guard > lst.shape[0]:
                raise RuntimeError("cycle in reference cell list")
        out[int(c)] = members
    return out


# ---------------------------------------------------------------- scenario I/O
def read_par(path) -> Config:
    """Minimal .par reader for test fixtures (src/io/ConfigReader.cpp:45-84
    keys that the simulation uses)."""
    keys = {"x_min": "x_min", "x_max": "x_max", "y_min": "y_min", "y_max": "y_max",
            "z_min": "z_min", "z_max": "z_max", "x_n": "x_n", "y_n": "y_n", "z_n": "z_n",
            "timestep_length": "timestep_length", "restdensity": "rest_density"}
    cfg = Config()
    for line in Path(path).read_text().splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0] in keys:
            setattr(cfg, keys[parts[0]], float(parts[1]))
    return cfg


def read_in(path):
    """(pos4, vel4) in the dumpData layout from a .in file
    (src/io/PartReader.cpp:35-91; pos.w = 0, vel.w = mass as in
    src/Simulation.cpp:120-134)."""
    lines = Path(path).read_text().splitlines()
    n = int(lines[0].split()[0])
    a = np.array([[_strtof(t) for t in l.split()[:7]] for l in lines[1:1 + n]], np.float32)
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    pos[:, :3] = a[:, 1:4]
    vel[:, :3] = a[:, 4:7]
    vel[:, 3] = a[:, 0]
    return pos, vel


_libc = C.CDLL(None)
_libc.strtof.restype = C.c_float
_libc.strtof.argtypes = [C.c_char_p, C.c_void_p]


def _strtof(text: str) -> float:
    """Decimal text to the nearest binary32, as istream >> float does."""
    return _libc.strtof(text.encode(), None)
