"""Synthetic scenes: seeded dam-break blocks with the benchmark shapes.

Every scene uses spacing 0.05 = h/2 with h = 0.1 (so the number density at
rest is 1/0.05^3 = 8000 per cubic metre: a fluid of 1000 kg/m^3 made of
particles of mass 1000*0.05^3 = 0.125 kg), gravity -9.81 along y, dt = 1/120,
4 solver iterations, relaxation epsilon 600, s_corr k = 0.1, n = 4,
dq = 0.2 h, XSPH c = 0.01 and vorticity epsilon 0.0005.  Each coordinate is
jittered by U(-0.01 spacing, +0.01 spacing) from the library's splitmix64
generator (seed 0x5EED unless given).

Block placement: the paper-mode walls sit h/4 inside the box, so a lattice
whose first particle is h/4 from the wall and whose extent is a whole number
of spacings fills the span between opposite walls exactly.  Blocks start at
the box minimum plus h/4 on every axis.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import MODE_PAPER, PARTICLE_DTYPE, Params, default_params, generate_block

H = 0.1
SPACING = 0.05
MASS = 1000.0 * SPACING ** 3
REST_DENSITY = 1.0 / SPACING ** 3
JITTER = 0.01 * SPACING
SEED = 0x5EED
DT = 1.0 / 120.0


@dataclass
class Scene:
    name: str
    params: Params
    particles: np.ndarray
    steps: int
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.particles.shape[0])


def base_params(box, cells, mode: int = MODE_PAPER) -> Params:
    p = default_params(mode)
    (p.x_min, p.y_min, p.z_min), (p.x_max, p.y_max, p.z_max) = (0.0, 0.0, 0.0), box
    p.x_n, p.y_n, p.z_n = cells
    p.time_step_length = DT
    p.rest_density = REST_DENSITY
    p.solver_iterations = 4
    p.relax_eps = 600.0
    p.scorr_k = 0.1
    p.scorr_n = 4
    p.scorr_dq = 0.2
    p.xsph_c = 0.01
    p.vort_eps = 0.0005
    p.gravity_y = -9.81
    p.wall_margin = 0.25 * H
    p.max_neighbours = 128
    return p


def block(origin, dims, seed: int) -> np.ndarray:
    nx, ny, nz = dims
    return generate_block(origin, nx, ny, nz, SPACING, JITTER, MASS, seed)


def dam_break(dims=(32, 32, 32), box=(1.6, 1.6, 3.2), seed: int = SEED, name: str = "dam_break") -> Scene:
    """One block in the box's minimum corner; cells of size h."""
    cells = tuple(int(round(b / H)) for b in box)
    p = base_params(box, cells)
    m = 0.25 * H
    ps = block((m, m, m), dims, seed)
    return Scene(name, p, ps, 500, {"block": list(dims), "box": list(box), "cells": list(cells),
                                    "origin": [m, m, m], "seed": seed})


def config_small(seed: int = SEED) -> Scene:
    """32,768 particles (32^3 block) in a 1.6 x 1.6 x 3.2 box, 500 steps."""
    return dam_break((32, 32, 32), (1.6, 1.6, 3.2), seed, "dam_break_32k")


def config_1m(seed: int = SEED) -> Scene:
    """1,048,576 particles (128 x 128 x 64 block) in a 6.4^3 box, 500 steps."""
    return dam_break((128, 128, 64), (6.4, 6.4, 6.4), seed, "single_scene_1m")


def config_4m(seed: int = SEED) -> Scene:
    """4,194,304 particles: two 128^3 blocks on the floor at opposite x ends of
    a 12.8 x 12.8 x 6.4 box, collapsing into each other; 200 steps."""
    box = (12.8, 12.8, 6.4)
    cells = (128, 128, 64)
    p = base_params(box, cells)
    m = 0.25 * H
    a = block((m, m, m), (128, 128, 128), seed)
    bx = box[0] - m - 127 * SPACING
    b = block((bx, m, m), (128, 128, 128), seed + 1)
    ps = np.concatenate([a, b])
    return Scene("double_dam_break_4m", p, ps, 200,
                 {"blocks": [[128, 128, 128]] * 2, "box": list(box), "cells": list(cells),
                  "origins": [[m, m, m], [bx, m, m]], "seed": seed})


def gen_grid(directory, name: str = "dam_coarse", h: float = 1.0, block_min=(10.0, 10.0, 10.0),
             block_max=(20.0, 20.0, 20.0), domain=(0.0, 30.0)):
    """The scenario pair tools/gen_grid.py writes (tools/gen_grid.py:1-49):
    a lattice of round(extent / s) + 1 particles per axis at spacing
    s = h / 2 from block_min (x outermost, unit mass, at rest) as <name>.in,
    and <name>.par with a cubic domain, h-sized cells, time_end 1,
    timestep 0.01 and restdensity = particles / block volume.  Returns the
    two paths."""
    from pathlib import Path

    from . import write_config, write_particles

    d = Path(directory)
    s = h / 2
    ext = [b - a for a, b in zip(block_min, block_max)]
    counts = [int(round(e / s)) + 1 for e in ext]
    ps = generate_block(block_min, *counts, s, 0.0, 1.0, 0)
    write_particles(d / f"{name}.in", ps)
    p = default_params()
    p.part_input_file = f"{name}.in".encode()
    p.time_end = 1.0
    p.time_step_length = 0.01
    p.x_min = p.y_min = p.z_min = domain[0]
    p.x_max = p.y_max = p.z_max = domain[1]
    p.x_n = p.y_n = p.z_n = float(int(round((domain[1] - domain[0]) / h)))
    p.rest_density = ps.shape[0] / (ext[0] * ext[1] * ext[2])
    write_config(d / f"{name}.par", p)
    return d / f"{name}.in", d / f"{name}.par"


def block_in_double_box(dims, seed: int, steps: int, name: str) -> Scene:
    """A dam-break block in the corner of a box twice the block's extent on
    every axis (rounded up to whole cells of size h)."""
    ext = [(d - 1) * SPACING + 2 * 0.25 * H for d in dims]
    cells = tuple(max(1, int(math.ceil(2 * e / H))) for e in ext)
    box = tuple(c * H for c in cells)
    p = base_params(box, cells)
    m = 0.25 * H
    ps = block((m, m, m), dims, seed)
    return Scene(name, p, ps, steps, {"block": list(dims), "box": list(box), "cells": list(cells),
                                      "seed": seed})


def _dims_for(n_target: float, ax: float, az: float):
    # block dims proportional to (ax, 1, az) with product ~ n_target
    base = (n_target / (ax * az)) ** (1.0 / 3.0)
    return tuple(max(2, int(round(v))) for v in (base * ax, base, base * az))


def mixed_batch(count: int = 256, n_min: int = 4096, n_max: int = 262144, seed: int = SEED) -> list[Scene]:
    """Independent dam breaks with log-uniform particle counts and block
    aspect ratios in [0.5, 2]; each box is twice the block extent."""
    rng = np.random.default_rng(seed)
    scenes = []
    for s in range(count):
        n_target = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        ax, az = rng.uniform(0.5, 2.0, size=2)
        scenes.append(block_in_double_box(_dims_for(n_target, ax, az), seed + 1000 + s, 300, f"batch_{s}"))
    return scenes


@dataclass
class Request:
    """One served scene solve: arrival time (s from the start of the stream),
    block dims, step count and seed; `scene()` builds the particles."""
    index: int
    arrival: float
    dims: tuple
    steps: int
    seed: int

    @property
    def n(self) -> int:
        return int(np.prod(self.dims))

    def scene(self) -> Scene:
        return block_in_double_box(self.dims, self.seed, self.steps, f"request_{self.index}")


def request_stream(duration_s: float, rate: float = 50.0, n_min: int = 8192, n_max: int = 524288,
                   steps_min: int = 100, steps_max: int = 1000, seed: int = SEED) -> list[Request]:
    """A seeded Poisson stream of dam-break solves: exponential inter-arrival
    times of mean 1/rate, N log-uniform in [n_min, n_max], block aspect
    ratios uniform in [0.5, 2], step counts uniform in {steps_min..steps_max}."""
    rng = np.random.default_rng(seed + 7)
    out = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration_s:
            break
        n_target = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        ax, az = rng.uniform(0.5, 2.0, size=2)
        steps = int(rng.integers(steps_min, steps_max + 1))
        i = len(out)
        out.append(Request(i, t, _dims_for(n_target, ax, az), steps, seed + 5000 + i))
    return out
