"""GB300 position-based-fluids step: Python host interface over the C-ABI.

The native library (``libpbf_gb300.so``, built by ``build.py`` from
``csrc/``) does all the work; this module only marshals arguments.  It
mirrors the reference's host interface (MrMagne/position-based-fluids):

* ``Simulation`` -- ``src/Simulation.hpp:41-108`` (init, initCells, step,
  dumpData, getters, setWaveGenerator);
* ``read_config`` / ``read_particles`` / ``data_path`` -- ConfigReader,
  PartReader and DataLoader (``src/io/*``, ``src/DataLoader.*``);
* ``op_*`` -- the neighbour-structure operators on device pointers;
* ``Batch`` / ``Server`` -- many scenes per step, and the request loop over
  them (no reference counterpart).

There is no CPU fallback: if the library is missing, importing this package
raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libpbf_gb300.so"

MODE_REF_COMPAT = 0
MODE_PAPER = 1

OK = 0
ERR_INVALID = 1
ERR_OOM = 2
ERR_CUDA = 3
ERR_DEVICE = 4
ERR_IO = 5
ERR_BUDGET = 6
ERR_STATE = 7
ERR_NOT_FOUND = 8

REQ_QUEUED = 0
REQ_ACTIVE = 1
REQ_DONE = 2


class Params(C.Structure):
    """pbf_params: ConfigParameters (src/Parameters.hpp:12-31) + solver settings."""

    _fields_ = [
        ("part_input_file", C.c_char * 256),
        ("time_step_length", C.c_float),
        ("time_end", C.c_float),
        ("part_out_freq", C.c_uint32),
        ("part_out_name_base", C.c_char * 256),
        ("vtk_out_freq", C.c_uint32),
        ("vtk_out_name_base", C.c_char * 256),
        ("cl_workgroup_1dsize", C.c_uint32),
        ("x_min", C.c_float), ("x_max", C.c_float),
        ("y_min", C.c_float), ("y_max", C.c_float),
        ("z_min", C.c_float), ("z_max", C.c_float),
        ("x_n", C.c_float), ("y_n", C.c_float), ("z_n", C.c_float),
        ("rest_density", C.c_float),
        ("mode", C.c_int32),
        ("solver_iterations", C.c_uint32),
        ("relax_eps", C.c_float),
        ("scorr_k", C.c_float),
        ("scorr_dq", C.c_float),
        ("scorr_n", C.c_int32),
        ("xsph_c", C.c_float),
        ("vort_eps", C.c_float),
        ("gravity_y", C.c_float),
        ("wall_margin", C.c_float),
        ("max_neighbours", C.c_uint32),
        ("grow_lists", C.c_uint32),
    ]

    @property
    def ncells(self) -> int:
        return int(self.x_n) * int(self.y_n) * int(self.z_n)

    @property
    def h(self) -> float:
        return float(np.float32(np.float32(self.x_max) - np.float32(self.x_min)) / np.float32(self.x_n))

    def copy(self) -> "Params":
        p = Params()
        C.pointer(p)[0] = self
        return p


class Particle(C.Structure):
    """pbf_particle: Particle (src/Particle.hpp:9-14)."""

    _fields_ = [("m", C.c_float), ("x", C.c_float * 3), ("v", C.c_float * 3), ("a", C.c_float * 3)]


PARTICLE_DTYPE = np.dtype([("m", np.float32), ("x", np.float32, 3), ("v", np.float32, 3),
                           ("a", np.float32, 3)])
assert PARTICLE_DTYPE.itemsize == C.sizeof(Particle)


class Camera(C.Structure):
    """pbf_camera: the reference's spherical camera (src/visual/visual.cpp:86-125)."""

    _fields_ = [("phi_deg", C.c_float), ("theta_deg", C.c_float), ("distance", C.c_float),
                ("target", C.c_float * 3), ("fovy_deg", C.c_float), ("znear", C.c_float),
                ("zfar", C.c_float), ("max_point_size", C.c_float)]


class Tuning(C.Structure):
    """pbf_tuning: launch shape of the gather passes (list build, fused list
    build + first lambda, lambda, delta-p, vorticity, XSPH)."""

    PASSES = ("nbr_build", "nbr_lambda", "lambda", "delta", "vorticity", "xsph_commit")
    _fields_ = [("threads", C.c_uint32 * 6), ("batch", C.c_uint32 * 6), ("fuse_first", C.c_uint32),
                ("trial_ms", C.c_float * 6), ("staged", C.c_uint32), ("radix_sort", C.c_uint32),
                ("masked_build", C.c_uint32)]

    def as_dict(self) -> dict:
        return {"threads": dict(zip(self.PASSES, self.threads)), "batch": dict(zip(self.PASSES, self.batch)),
                "fuse_first": int(self.fuse_first), "staged": int(self.staged),
                "radix_sort": int(self.radix_sort), "masked_build": int(self.masked_build),
                "trial_ms": dict(zip(self.PASSES, self.trial_ms))}


class ServerStats(C.Structure):
    """pbf_server_stats."""

    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("batch_steps", C.c_uint64), ("particle_steps", C.c_uint64),
                ("queued", C.c_uint32), ("active", C.c_uint32),
                ("active_particles", C.c_uint32), ("active_cells", C.c_uint32),
                ("max_particles", C.c_uint32), ("max_cells", C.c_uint32), ("max_scenes", C.c_uint32),
                ("pad_", C.c_uint32), ("device_bytes", C.c_uint64), ("launches", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad_"}


_lib = None


class PbfError(RuntimeError):
    def __init__(self, status: int, what: str):
        msg = f"{what}: {_lib.pbf_status_string(status).decode()}"
        detail = _lib.pbf_last_error_message().decode()
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)
        self.status = status


def lib():
    """The loaded native library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(str(LIB_PATH))
        vp, u32, f32, i32 = C.c_void_p, C.c_uint32, C.c_float, C.c_int
        pp = C.POINTER(Params)
        sig = {
            "pbf_abi_version": ([], i32),
            "pbf_status_string": ([i32], C.c_char_p),
            "pbf_last_error_message": ([], C.c_char_p),
            "pbf_params_default": ([pp], None),
            "pbf_read_config": ([C.c_char_p, pp], i32),
            "pbf_read_particles": ([C.c_char_p, C.POINTER(vp), C.POINTER(u32)], i32),
            "pbf_free": ([vp], None),
            "pbf_write_particles": ([C.c_char_p, vp, u32], i32),
            "pbf_write_particles_bin": ([C.c_char_p, vp, u32], i32),
            "pbf_write_config": ([C.c_char_p, pp], i32),
            "pbf_write_vtk": ([C.c_char_p, vp, vp, u32], i32),
            "pbf_data_path": ([C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t], i32),
            "pbf_generate_block": ([vp, u32, u32, u32, f32, f32, f32, C.c_uint64, vp], i32),
            "pbf_create": ([pp, vp, u32, C.POINTER(vp)], i32),
            "pbf_init": ([vp], i32),
            "pbf_init_cells": ([vp], i32),
            "pbf_step": ([vp, u32], i32),
            "pbf_sync": ([vp], i32),
            "pbf_dump_data": ([vp, vp, vp], i32),
            "pbf_set_state": ([vp, vp, vp], i32),
            "pbf_set_state_async": ([vp, vp, vp], i32),
            "pbf_dump_data_async": ([vp, vp, vp], i32),
            "pbf_host_alloc": ([C.c_size_t, C.POINTER(vp)], i32),
            "pbf_host_free": ([vp], i32),
            "pbf_set_wave": ([vp, f32], i32),
            "pbf_get_num_particles": ([vp, C.POINTER(u32)], i32),
            "pbf_get_sizes": ([vp, vp, vp], i32),
            "pbf_get_stream": ([vp, C.POINTER(vp)], i32),
            "pbf_set_stage_timing": ([vp, i32], i32),
            "pbf_stage_times": ([vp, vp], i32),
            "pbf_kernel_times": ([vp, u32, vp, vp, vp, C.POINTER(u32)], i32),
            "pbf_set_graph": ([vp, i32], i32),
            "pbf_launches_per_step": ([vp, C.POINTER(u32)], i32),
            "pbf_get_density": ([vp, vp], i32),
            "pbf_neighbour_stats": ([vp, C.POINTER(u32), C.POINTER(u32)], i32),
            "pbf_tile_stats": ([vp, C.POINTER(u32), C.POINTER(u32)], i32),
            "pbf_list_capacity": ([vp, C.POINTER(u32), C.POINTER(u32)], i32),
            "pbf_get_cells": ([vp, vp, vp, vp], i32),
            "pbf_destroy": ([vp], i32),
            "pbf_autotune": ([vp, u32, C.POINTER(Tuning)], i32),
            "pbf_camera_default": ([pp, C.POINTER(Camera)], None),
            "pbf_render": ([vp, C.POINTER(Camera), u32, u32, vp], i32),
            "pbf_batch_render_scene": ([vp, u32, C.POINTER(Camera), u32, u32, vp], i32),
            "pbf_get_tuning": ([vp, C.POINTER(Tuning)], i32),
            "pbf_set_tuning": ([vp, C.POINTER(Tuning)], i32),
            "pbf_batch_autotune": ([vp, u32, C.POINTER(Tuning)], i32),
            "pbf_batch_get_tuning": ([vp, C.POINTER(Tuning)], i32),
            "pbf_batch_set_tuning": ([vp, C.POINTER(Tuning)], i32),
            "pbf_op_cell_hash": ([pp, vp, u32, vp, vp], i32),
            "pbf_op_sort_scratch_bytes": ([u32, u32], C.c_size_t),
            "pbf_op_sort_pairs": ([vp, vp, u32, u32, vp, vp, vp, C.c_size_t, vp], i32),
            "pbf_op_sort_status": ([vp, u32, u32, vp], i32),
            "pbf_op_sort_pairs_noalloc": ([vp, vp, u32, u32, vp, vp, vp, vp], i32),
            "pbf_op_sort_cells_scratch_bytes": ([u32, u32], C.c_size_t),
            "pbf_op_sort_cells": ([vp, u32, u32, vp, vp, vp, vp, C.c_size_t, vp], i32),
            "pbf_op_sort_cells_status": ([vp, u32, u32, vp], i32),
            "pbf_op_cell_offsets": ([vp, u32, u32, vp, vp], i32),
            "pbf_op_find_cells": ([vp, u32, vp, vp], i32),
            "pbf_selftest_bounded_wait": ([u32, C.POINTER(u32)], i32),
            "pbf_batch_create": ([pp, u32, u32, u32, C.POINTER(vp)], i32),
            "pbf_batch_device_bytes": ([pp, u32, u32, u32], C.c_size_t),
            "pbf_batch_add_scene": ([vp, pp, vp, u32, C.POINTER(u32)], i32),
            "pbf_batch_remove_scene": ([vp, u32], i32),
            "pbf_batch_step": ([vp, u32], i32),
            "pbf_batch_sync": ([vp], i32),
            "pbf_batch_dump_scene": ([vp, u32, vp, vp], i32),
            "pbf_batch_set_wave": ([vp, u32, f32], i32),
            "pbf_batch_info": ([vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)], i32),
            "pbf_batch_get_stream": ([vp, C.POINTER(vp)], i32),
            "pbf_batch_launches_per_step": ([vp, C.POINTER(u32)], i32),
            "pbf_batch_neighbour_stats": ([vp, C.POINTER(u32), C.POINTER(u32)], i32),
            "pbf_batch_destroy": ([vp], i32),
            "pbf_server_create": ([pp, C.c_uint64, u32, f32, u32, C.POINTER(vp)], i32),
            "pbf_server_submit": ([vp, pp, vp, u32, u32, C.POINTER(C.c_uint64)], i32),
            "pbf_server_poll": ([vp, i32, vp, u32, C.POINTER(u32), C.POINTER(i32)], i32),
            "pbf_server_request_info": ([vp, C.c_uint64, C.POINTER(i32), C.POINTER(u32), C.POINTER(u32)],
                                        i32),
            "pbf_server_result": ([vp, C.c_uint64, vp, vp], i32),
            "pbf_server_stats_get": ([vp, C.POINTER(ServerStats)], i32),
            "pbf_server_destroy": ([vp], i32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def exported_symbols() -> list[str]:
    """Names of every pbf_* function this binding declares."""
    lib()
    return [n for n in dir(_lib) if n.startswith("pbf_")]


def _check(status: int, what: str) -> None:
    if status != OK:
        raise PbfError(status, what)


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


# ------------------------------------------------------------- scenario layer
def default_params(mode: int = MODE_PAPER) -> Params:
    p = Params()
    lib().pbf_params_default(C.byref(p))
    p.mode = mode
    return p


def read_config(path, base: Params | None = None) -> Params:
    p = base.copy() if base is not None else default_params()
    _check(lib().pbf_read_config(str(path).encode(), C.byref(p)), "read_config")
    return p


def read_particles(path) -> np.ndarray:
    """Particles of a .in file as a structured array (PARTICLE_DTYPE)."""
    buf = C.c_void_p()
    n = C.c_uint32()
    _check(lib().pbf_read_particles(str(path).encode(), C.byref(buf), C.byref(n)), "read_particles")
    out = np.zeros(n.value, PARTICLE_DTYPE)
    if n.value:
        C.memmove(out.ctypes.data, buf, n.value * PARTICLE_DTYPE.itemsize)
        lib().pbf_free(buf)
    return out


def write_particles(path, particles: np.ndarray, binary: bool = False) -> None:
    """A .in file (text, the reference's PartReader format) or, with
    binary=True, the binary particle format read_particles also accepts."""
    ps = np.ascontiguousarray(particles, PARTICLE_DTYPE)
    fn = lib().pbf_write_particles_bin if binary else lib().pbf_write_particles
    _check(fn(str(path).encode(), _ptr(ps), int(ps.shape[0])), "write_particles")


def write_config(path, params: Params) -> None:
    """A .par file with every key (reference keys and extension keys)."""
    _check(lib().pbf_write_config(str(path).encode(), C.byref(params)), "write_config")


def write_vtk(path, pos4: np.ndarray, vel4: np.ndarray) -> None:
    """Legacy binary VTK POLYDATA of dumpData-layout arrays."""
    pos = np.ascontiguousarray(pos4, np.float32).reshape(-1, 4)
    vel = np.ascontiguousarray(vel4, np.float32).reshape(-1, 4)
    _check(lib().pbf_write_vtk(str(path).encode(), _ptr(pos), _ptr(vel), int(pos.shape[0])), "write_vtk")


def data_path(root, kind: str, name: str) -> str:
    buf = C.create_string_buffer(4096)
    _check(lib().pbf_data_path(str(root).encode(), kind.encode(), name.encode(), buf, 4096), "data_path")
    return buf.value.decode()


def generate_block(origin, nx: int, ny: int, nz: int, spacing: float, jitter: float, mass: float,
                   seed: int) -> np.ndarray:
    out = np.zeros(nx * ny * nz, PARTICLE_DTYPE)
    o = np.asarray(origin, np.float32)
    _check(lib().pbf_generate_block(_ptr(o), nx, ny, nz, spacing, jitter, mass, seed & (2**64 - 1),
                                    _ptr(out)), "generate_block")
    return out


def particles_from_state(pos4: np.ndarray, vel4: np.ndarray) -> np.ndarray:
    """Particles from dumpData-layout arrays (vel.w = mass)."""
    pos4 = np.asarray(pos4, np.float32).reshape(-1, 4)
    vel4 = np.asarray(vel4, np.float32).reshape(-1, 4)
    out = np.zeros(pos4.shape[0], PARTICLE_DTYPE)
    out["m"] = vel4[:, 3]
    out["x"] = pos4[:, :3]
    out["v"] = vel4[:, :3]
    return out


def state_from_particles(ps: np.ndarray):
    """(pos4, vel4) in the dumpData layout before the first step."""
    n = ps.shape[0]
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    pos[:, :3] = ps["x"]
    vel[:, :3] = ps["v"]
    vel[:, 3] = ps["m"]
    return pos, vel


# --------------------------------------------------------------- Simulation
class Simulation:
    """The reference's Simulation (src/Simulation.hpp:41-108) on one GB300."""

    def __init__(self, params: Params, particles: np.ndarray):
        self.params = params.copy()
        self._particles = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        self.n = int(self._particles.shape[0])
        h = C.c_void_p()
        _check(lib().pbf_create(C.byref(self.params), _ptr(self._particles), self.n, C.byref(h)), "pbf_create")
        self._h = h

    # lifecycle ------------------------------------------------------------
    def init(self):
        _check(lib().pbf_init(self._h), "pbf_init")

    def initCells(self):  # noqa: N802 (reference name)
        _check(lib().pbf_init_cells(self._h), "pbf_init_cells")

    def step(self, nsteps: int = 1, sync: bool = True):
        _check(lib().pbf_step(self._h, nsteps), "pbf_step")
        if sync:
            self.sync()

    def sync(self):
        _check(lib().pbf_sync(self._h), "pbf_sync")

    def close(self):
        if getattr(self, "_h", None):
            lib().pbf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # state ------------------------------------------------------------------
    def dumpData(self):  # noqa: N802 (reference name)
        pos = np.zeros((self.n, 4), np.float32)
        vel = np.zeros((self.n, 4), np.float32)
        _check(lib().pbf_dump_data(self._h, _ptr(pos), _ptr(vel)), "pbf_dump_data")
        return pos, vel

    def set_state(self, pos4, vel4):
        pos = np.ascontiguousarray(pos4, np.float32).reshape(self.n, 4)
        vel = np.ascontiguousarray(vel4, np.float32).reshape(self.n, 4)
        _check(lib().pbf_set_state(self._h, _ptr(pos), _ptr(vel)), "pbf_set_state")

    def save_state(self, path):
        """Checkpoint: the state in the dumpData layout, as an .npz file."""
        pos, vel = self.dumpData()
        np.savez(path, pos=pos, vel=vel, n=self.n)

    def load_state(self, path):
        """Resumes from a checkpoint written by save_state."""
        d = np.load(path)
        if int(d["n"]) != self.n:
            raise PbfError(ERR_INVALID, "load_state: particle count differs")
        self.set_state(d["pos"], d["vel"])

    def set_state_async(self, pos_ptr: int, vel_ptr: int):
        _check(lib().pbf_set_state_async(self._h, pos_ptr, vel_ptr), "pbf_set_state_async")

    def dump_data_async(self, pos_ptr: int, vel_ptr: int):
        _check(lib().pbf_dump_data_async(self._h, pos_ptr, vel_ptr), "pbf_dump_data_async")

    def density(self) -> np.ndarray:
        out = np.zeros(self.n, np.float32)
        _check(lib().pbf_get_density(self._h, _ptr(out)), "pbf_get_density")
        return out

    def neighbour_stats(self) -> tuple[int, int]:
        """(largest neighbour count, particles over the list capacity) of the
        last step's neighbour lists."""
        mx, over = C.c_uint32(), C.c_uint32()
        _check(lib().pbf_neighbour_stats(self._h, C.byref(mx), C.byref(over)), "pbf_neighbour_stats")
        return mx.value, over.value

    def list_capacity(self) -> tuple[int, int]:
        """(neighbour-list capacity in use, times it has grown)."""
        cap, grows = C.c_uint32(), C.c_uint32()
        _check(lib().pbf_list_capacity(self._h, C.byref(cap), C.byref(grows)), "pbf_list_capacity")
        return int(cap.value), int(grows.value)

    def tile_stats(self) -> tuple[int, int]:
        """(staged, unstaged) 128-slot tiles of the last step's staged passes."""
        a, b = C.c_uint32(), C.c_uint32()
        _check(lib().pbf_tile_stats(self._h, C.byref(a), C.byref(b)), "pbf_tile_stats")
        return int(a.value), int(b.value)

    def cells(self):
        """(hash per particle, sorted permutation, inclusive ranges per cell)."""
        hsh = np.zeros(self.n, np.uint32)
        perm = np.zeros(self.n, np.uint32)
        rng = np.zeros((self.params.ncells, 2), np.int32)
        _check(lib().pbf_get_cells(self._h, _ptr(hsh), _ptr(perm), _ptr(rng)), "pbf_get_cells")
        return hsh, perm, rng

    # getters / setters ----------------------------------------------------------
    def getNumberParticles(self) -> int:  # noqa: N802
        n = C.c_uint32()
        _check(lib().pbf_get_num_particles(self._h, C.byref(n)), "pbf_get_num_particles")
        return n.value

    def getSizesMin(self):  # noqa: N802
        mn = np.zeros(4, np.float32)
        mx = np.zeros(4, np.float32)
        _check(lib().pbf_get_sizes(self._h, _ptr(mn), _ptr(mx)), "pbf_get_sizes")
        return mn

    def getSizesMax(self):  # noqa: N802
        mn = np.zeros(4, np.float32)
        mx = np.zeros(4, np.float32)
        _check(lib().pbf_get_sizes(self._h, _ptr(mn), _ptr(mx)), "pbf_get_sizes")
        return mx

    def setWaveGenerator(self, value: float):  # noqa: N802
        _check(lib().pbf_set_wave(self._h, float(value)), "pbf_set_wave")

    def stream(self) -> int:
        s = C.c_void_p()
        _check(lib().pbf_get_stream(self._h, C.byref(s)), "pbf_get_stream")
        return s.value or 0

    def set_stage_timing(self, enable: bool):
        _check(lib().pbf_set_stage_timing(self._h, int(enable)), "pbf_set_stage_timing")

    def stage_times(self) -> np.ndarray:
        ms = np.zeros(4, np.float32)
        _check(lib().pbf_stage_times(self._h, _ptr(ms)), "pbf_stage_times")
        return ms

    def kernel_times(self) -> dict:
        """{kernel name: (total ms, launches)} since timing was enabled."""
        cnt = C.c_uint32()
        _check(lib().pbf_kernel_times(self._h, 0, None, None, None, C.byref(cnt)), "pbf_kernel_times")
        cap = cnt.value
        names = C.create_string_buffer(32 * max(cap, 1))
        ms = np.zeros(max(cap, 1), np.float32)
        la = np.zeros(max(cap, 1), np.uint32)
        _check(lib().pbf_kernel_times(self._h, cap, names, _ptr(ms), _ptr(la), C.byref(cnt)), "pbf_kernel_times")
        out = {}
        for q in range(min(cap, cnt.value)):
            nm = names.raw[32 * q:32 * q + 32].split(b"\0", 1)[0].decode()
            out[nm] = (float(ms[q]), int(la[q]))
        return out

    def set_graph(self, enable: bool):
        _check(lib().pbf_set_graph(self._h, int(enable)), "pbf_set_graph")

    def render(self, camera: Camera | None = None, width: int = 640, height: int = 480) -> np.ndarray:
        """The current state drawn as the reference's renderer draws it:
        (height, width, 3) uint8, top row first."""
        cam = camera if camera is not None else default_camera(self.params)
        img = np.zeros((height, width, 3), np.uint8)
        _check(lib().pbf_render(self._h, C.byref(cam), width, height, _ptr(img)), "pbf_render")
        return img

    def autotune(self, trial_steps: int = 3) -> Tuning:
        """Picks the fastest launch shape of each gather pass on this scene
        (the state is restored; results are unchanged)."""
        t = Tuning()
        _check(lib().pbf_autotune(self._h, trial_steps, C.byref(t)), "pbf_autotune")
        return t

    def tuning(self) -> Tuning:
        t = Tuning()
        _check(lib().pbf_get_tuning(self._h, C.byref(t)), "pbf_get_tuning")
        return t

    def set_tuning(self, t: Tuning):
        _check(lib().pbf_set_tuning(self._h, C.byref(t)), "pbf_set_tuning")

    def launches_per_step(self) -> int:
        n = C.c_uint32()
        _check(lib().pbf_launches_per_step(self._h, C.byref(n)), "pbf_launches_per_step")
        return n.value


class Batch:
    """Many paper-mode scenes advanced together (pbf_batch_* in include/pbf.h).

    `solver` carries the shared solver settings (h, iterations, s_corr,
    XSPH, vorticity); each scene brings its own box, grid and walls."""

    def __init__(self, solver: Params, max_scenes: int, max_particles: int, max_cells: int):
        self.solver = solver.copy()
        h = C.c_void_p()
        _check(lib().pbf_batch_create(C.byref(self.solver), max_scenes, max_particles, max_cells, C.byref(h)),
               "pbf_batch_create")
        self._h = h
        self._n = {}

    @staticmethod
    def device_bytes(solver: Params, max_scenes: int, max_particles: int, max_cells: int) -> int:
        return int(lib().pbf_batch_device_bytes(C.byref(solver), max_scenes, max_particles, max_cells))

    def add_scene(self, params: Params, particles: np.ndarray) -> int:
        ps = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        sid = C.c_uint32()
        _check(lib().pbf_batch_add_scene(self._h, C.byref(params), _ptr(ps), int(ps.shape[0]), C.byref(sid)),
               "pbf_batch_add_scene")
        self._n[sid.value] = int(ps.shape[0])
        return sid.value

    def remove_scene(self, scene_id: int):
        _check(lib().pbf_batch_remove_scene(self._h, scene_id), "pbf_batch_remove_scene")
        self._n.pop(scene_id, None)

    def step(self, nsteps: int = 1, sync: bool = True):
        _check(lib().pbf_batch_step(self._h, nsteps), "pbf_batch_step")
        if sync:
            self.sync()

    def sync(self):
        _check(lib().pbf_batch_sync(self._h), "pbf_batch_sync")

    def dump_scene(self, scene_id: int):
        n = self._n.get(scene_id)
        if n is None:
            raise PbfError(ERR_NOT_FOUND, "pbf_batch_dump_scene")
        pos = np.zeros((n, 4), np.float32)
        vel = np.zeros((n, 4), np.float32)
        _check(lib().pbf_batch_dump_scene(self._h, scene_id, _ptr(pos), _ptr(vel)), "pbf_batch_dump_scene")
        return pos, vel

    def set_wave(self, scene_id: int, value: float):
        _check(lib().pbf_batch_set_wave(self._h, scene_id, float(value)), "pbf_batch_set_wave")

    def info(self):
        """(scenes, particles, cells) currently held."""
        s, p, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        _check(lib().pbf_batch_info(self._h, C.byref(s), C.byref(p), C.byref(c)), "pbf_batch_info")
        return s.value, p.value, c.value

    def stream(self) -> int:
        s = C.c_void_p()
        _check(lib().pbf_batch_get_stream(self._h, C.byref(s)), "pbf_batch_get_stream")
        return s.value or 0

    def launches_per_step(self) -> int:
        n = C.c_uint32()
        _check(lib().pbf_batch_launches_per_step(self._h, C.byref(n)), "pbf_batch_launches_per_step")
        return n.value

    def neighbour_stats(self) -> tuple[int, int]:
        """(largest neighbour count, particles over the list capacity) of the
        last step's neighbour lists, over every scene."""
        mx, over = C.c_uint32(), C.c_uint32()
        _check(lib().pbf_batch_neighbour_stats(self._h, C.byref(mx), C.byref(over)),
               "pbf_batch_neighbour_stats")
        return mx.value, over.value

    def autotune(self, trial_steps: int = 3) -> Tuning:
        t = Tuning()
        _check(lib().pbf_batch_autotune(self._h, trial_steps, C.byref(t)), "pbf_batch_autotune")
        return t

    def render_scene(self, scene_id: int, params: Params, camera: Camera | None = None,
                     width: int = 640, height: int = 480) -> np.ndarray:
        cam = camera if camera is not None else default_camera(params)
        img = np.zeros((height, width, 3), np.uint8)
        _check(lib().pbf_batch_render_scene(self._h, scene_id, C.byref(cam), width, height, _ptr(img)),
               "pbf_batch_render_scene")
        return img

    def tuning(self) -> Tuning:
        t = Tuning()
        _check(lib().pbf_batch_get_tuning(self._h, C.byref(t)), "pbf_batch_get_tuning")
        return t

    def set_tuning(self, t: Tuning):
        _check(lib().pbf_batch_set_tuning(self._h, C.byref(t)), "pbf_batch_set_tuning")

    def close(self):
        if getattr(self, "_h", None):
            lib().pbf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """Served scenes (pbf_server_* in include/pbf.h): a request loop with
    continuous batching over one batch sized by an HBM budget."""

    def __init__(self, solver: Params, hbm_budget_bytes: int, max_scenes: int = 1024,
                 cells_per_particle: float = 2.0, max_chunk: int = 16):
        self.solver = solver.copy()
        h = C.c_void_p()
        _check(lib().pbf_server_create(C.byref(self.solver), int(hbm_budget_bytes), max_scenes,
                                       float(cells_per_particle), max_chunk, C.byref(h)), "pbf_server_create")
        self._h = h
        self._n = {}
        self._ids = (C.c_uint64 * 4096)()

    def submit(self, params: Params, particles: np.ndarray, steps: int) -> int:
        ps = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        rid = C.c_uint64()
        _check(lib().pbf_server_submit(self._h, C.byref(params), _ptr(ps), int(ps.shape[0]), int(steps),
                                       C.byref(rid)), "pbf_server_submit")
        self._n[rid.value] = int(ps.shape[0])
        return rid.value

    def poll(self, wait: bool = False):
        """One turn of the loop: (ids completed in this turn, busy)."""
        cnt = C.c_uint32()
        busy = C.c_int()
        _check(lib().pbf_server_poll(self._h, int(wait), self._ids, len(self._ids), C.byref(cnt),
                                     C.byref(busy)), "pbf_server_poll")
        return [self._ids[i] for i in range(min(cnt.value, len(self._ids)))], bool(busy.value)

    def run_until_idle(self):
        done = []
        busy = True
        while busy:
            ids, busy = self.poll(wait=True)
            done += ids
        return done

    def info(self, rid: int):
        """(state, particles, steps done) of a request."""
        st, n, k = C.c_int(), C.c_uint32(), C.c_uint32()
        _check(lib().pbf_server_request_info(self._h, rid, C.byref(st), C.byref(n), C.byref(k)),
               "pbf_server_request_info")
        return st.value, n.value, k.value

    def result(self, rid: int):
        n = self._n.get(rid, 1)
        pos = np.zeros((n, 4), np.float32)
        vel = np.zeros((n, 4), np.float32)
        _check(lib().pbf_server_result(self._h, rid, _ptr(pos), _ptr(vel)), "pbf_server_result")
        self._n.pop(rid, None)
        return pos, vel

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().pbf_server_stats_get(self._h, C.byref(st)), "pbf_server_stats_get")
        return st.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            lib().pbf_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def default_camera(params: Params) -> Camera:
    """The reference's initial camera for the box of `params`."""
    cam = Camera()
    lib().pbf_camera_default(C.byref(params), C.byref(cam))
    return cam


def write_ppm(path, img: np.ndarray) -> None:
    """Binary PPM (P6) of an (H, W, 3) uint8 image."""
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(img, np.uint8).tobytes())


# ------------------------------------------------------------------ operators
def op_cell_hash(params: Params, d_pred4: int, n: int, d_hash: int, stream: int = 0):
    _check(lib().pbf_op_cell_hash(C.byref(params), d_pred4, n, d_hash, stream), "pbf_op_cell_hash")


def op_sort_scratch_bytes(n: int, key_bits: int) -> int:
    return int(lib().pbf_op_sort_scratch_bytes(n, key_bits))


def op_sort_pairs(d_keys_in: int, d_vals_in, n: int, key_bits: int, d_keys_out: int, d_vals_out: int,
                  d_scratch: int, scratch_bytes: int, stream: int = 0):
    _check(lib().pbf_op_sort_pairs(d_keys_in, d_vals_in, n, key_bits, d_keys_out, d_vals_out, d_scratch,
                                   scratch_bytes, stream), "pbf_op_sort_pairs")


def op_sort_status(d_scratch: int, n: int, key_bits: int, stream: int = 0):
    _check(lib().pbf_op_sort_status(d_scratch, n, key_bits, stream), "pbf_op_sort_status")


def op_sort_cells_scratch_bytes(n: int, ncells: int) -> int:
    return int(lib().pbf_op_sort_cells_scratch_bytes(n, ncells))


def op_sort_cells(d_keys: int, n: int, ncells: int, d_offsets: int, d_sorted_keys: int, d_perm: int,
                  d_scratch: int, scratch_bytes: int, stream: int = 0):
    _check(lib().pbf_op_sort_cells(d_keys, n, ncells, d_offsets, d_sorted_keys, d_perm, d_scratch,
                                   scratch_bytes, stream), "pbf_op_sort_cells")


def op_sort_cells_status(d_scratch: int, n: int, ncells: int, stream: int = 0):
    _check(lib().pbf_op_sort_cells_status(d_scratch, n, ncells, stream), "pbf_op_sort_cells_status")


def op_cell_offsets(d_sorted_keys: int, n: int, ncells: int, d_offsets: int, stream: int = 0):
    _check(lib().pbf_op_cell_offsets(d_sorted_keys, n, ncells, d_offsets, stream), "pbf_op_cell_offsets")


def op_find_cells(d_offsets: int, ncells: int, d_first_last: int, stream: int = 0):
    _check(lib().pbf_op_find_cells(d_offsets, ncells, d_first_last, stream), "pbf_op_find_cells")


from . import scenes  # noqa: E402  (needs the definitions above)
