"""Staged cell blocks (tuning staged = 1, pbf_tile.cu) against the L1 gather
passes.

Statement: the staged passes visit each particle's neighbours in the same
order with the same arithmetic, so a step gives the SAME BITS as the L1
passes -- in blocks that stage their neighbourhood, in blocks that do not
(more than 3072 candidates in the halo), for particles that re-derive their
sets (lists capped at 16 entries), in sparse scenes, in a batch of mixed
scenes, and against the FP64 oracle within the 1e-5 h bound.
"""
from __future__ import annotations

import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def staged_tuning(sim, on: bool):
    t = sim.tuning()
    t.staged = 1 if on else 0
    return t


def run(pbf, params, particles, steps, staged):
    with pbf.Simulation(params, particles) as sim:
        sim.init()
        sim.set_tuning(staged_tuning(sim, staged))
        sim.step(steps)
        out = sim.dumpData()
        dens = sim.density()
        tiles = sim.tile_stats()
        lists = sim.neighbour_stats()
    return out, dens, tiles, lists


def assert_same(a, b, what):
    (pa, va), da = a[0], a[1]
    (pb, vb), db = b[0], b[1]
    assert np.array_equal(bits(pa), bits(pb)), f"{what}: positions"
    assert np.array_equal(bits(va), bits(vb)), f"{what}: velocities"
    assert np.array_equal(bits(da), bits(db)), f"{what}: densities"


def scattered(pbf, n, box, seed):
    """Particles spread thinly over a large box (most cells empty)."""
    rng = np.random.default_rng(seed)
    cells = tuple(int(round(b / pbf.scenes.H)) for b in box)
    p = pbf.scenes.base_params(box, cells)
    ps = np.zeros(n, pbf.PARTICLE_DTYPE)
    lo = 0.3 * pbf.scenes.H
    ps["x"] = rng.uniform(lo, np.array(box) - lo, size=(n, 3)).astype(np.float32)
    ps["m"] = pbf.scenes.MASS
    return p, ps


def dense_block(pbf, seed):
    """A block at a quarter of the usual spacing (64 particles per cell, with
    the rest density to match, so it stays that dense): a cell block's halo
    holds far more than 3072 candidates, so it is not staged."""
    dims = (16, 16, 16)
    box = (1.6, 1.6, 1.6)
    cells = tuple(int(round(b / pbf.scenes.H)) for b in box)
    p = pbf.scenes.base_params(box, cells)
    p.rest_density = 1.0 / 0.025 ** 3
    p.max_neighbours = 512
    ps = pbf.generate_block((0.5, 0.5, 0.5), *dims, 0.025, 0.0002, pbf.scenes.MASS / 64, seed)
    return p, ps


@pytest.mark.parametrize("case", ["dam_break", "capped_lists", "scattered", "dense"])
def test_staged_equals_l1_gathers(pbf, case):
    if case in ("dam_break", "capped_lists"):
        sc = pbf.scenes.dam_break((24, 20, 16), (1.6, 1.6, 1.6), seed=41)
        params, particles = sc.params.copy(), sc.particles
        if case == "capped_lists":
            params.max_neighbours = 16
            params.grow_lists = 0
    elif case == "scattered":
        params, particles = scattered(pbf, 6000, (3.2, 3.2, 3.2), 42)
    else:
        params, particles = dense_block(pbf, 43)
    steps = 2 if case == "dense" else 6  # the overdense block spreads out within a few steps
    l1 = run(pbf, params, particles, steps, False)
    st = run(pbf, params, particles, steps, True)
    assert_same(st, l1, case)
    assert st[3] == l1[3]  # same neighbour counts
    staged, unstaged = st[2]
    if case == "dense":
        assert unstaged > 0, st[2]
    else:
        assert staged > 0 and unstaged == 0, st[2]
    if case == "capped_lists":
        assert st[3][1] > 0  # some particles re-derive their sets
    assert l1[2] == (0, 0)


def test_staged_batch_equals_l1_batch(pbf):
    scenes = pbf.scenes.mixed_batch(count=6, n_min=1000, n_max=30000, seed=44)
    cap = (len(scenes), sum(s.n for s in scenes), sum(s.params.ncells for s in scenes))
    out = []
    for staged in (False, True):
        with pbf.Batch(scenes[0].params, *cap) as b:
            ids = [b.add_scene(s.params, s.particles) for s in scenes]
            t = b.tuning()
            t.staged = 1 if staged else 0
            b.set_tuning(t)
            b.step(6)
            out.append([b.dump_scene(i) for i in ids])
    for s, x, y in zip(scenes, *out):
        for a, c in zip(x, y):
            assert np.array_equal(bits(a), bits(c)), s.name


def test_staged_step_vs_fp64_oracle(pbf, oracle_mod):
    sc = pbf.scenes.dam_break((20, 20, 20), (1.6, 1.6, 1.6), seed=45)
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        sim.set_tuning(staged_tuning(sim, True))
        sim.step(8)
        pos, vel = sim.dumpData()
        sim.set_state(pos, vel)
        sim.step(1)
        gp, gv = sim.dumpData()
        assert sim.tile_stats()[0] > 0
    prm = ge.paper_params_for_oracle(sc.params)
    op, ov, *_ = oracle_mod.paper_steps_f64(prm, pos.astype(np.float64), vel.astype(np.float64), 1)
    h = sc.params.h
    assert np.abs(gp[:, :3].astype(np.float64) - op[:, :3]).max() <= 1e-5 * h
    vmax = np.abs(ov[:, :3]).max()
    assert np.abs(gv[:, :3].astype(np.float64) - ov[:, :3]).max() <= 1e-3 + 1e-4 * vmax


def test_tuner_keeps_bits_with_staged_candidates(pbf):
    sc = pbf.scenes.dam_break((20, 20, 10), (1.6, 1.6, 0.8), seed=46)
    ref = run(pbf, sc.params, sc.particles, 8, False)
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        sim.step(2)
        t = sim.autotune(2).as_dict()
        assert t["staged"] in (0, 1)
        sim.step(6)
        got = (sim.dumpData(), sim.density())
    assert_same(got, ref, "tuned")
