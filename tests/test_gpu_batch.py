"""Batched scenes (pbf_batch_*): many paper-mode scenes in one step.

Equality statement (checked below): a scene's positions and velocities after
K steps in a batch are BIT-IDENTICAL to

  * the same scene run alone through the plain simulation (pbf_sim), when the
    scene's cell length equals the batch's h exactly;
  * the same scene run alone in a batch of one, for any scene;

whatever other scenes share the batch, and across removals and additions of
other scenes between steps.  The scene ranges of the sorted state never mix
(keys are scene-major) and every kernel works on one particle per thread with
neighbours from its own scene, so every particle runs the same instructions
on the same operands.
"""
from __future__ import annotations

import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu

POS_TOL_H = 1e-5


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def plain_scenes(pbf):
    """Scenes whose cell length is exactly h = 0.1 (extents 0.1 x 2^k)."""
    dam = pbf.scenes.dam_break
    return [dam((12, 10, 14), (1.6, 1.6, 1.6), seed=11, name="a"),
            dam((20, 16, 8), (1.6, 1.6, 0.8), seed=12, name="b"),
            dam((6, 6, 6), (0.8, 0.8, 0.8), seed=13, name="c"),
            dam((24, 12, 12), (3.2, 1.6, 1.6), seed=14, name="d")]


def capacity(scenes):
    return (len(scenes), sum(s.n for s in scenes), sum(s.params.ncells for s in scenes))


def run_plain(pbf, scene, steps, wave=None):
    with pbf.Simulation(scene.params, scene.particles) as sim:
        sim.init()
        if wave is not None:
            sim.setWaveGenerator(wave)
        sim.step(steps)
        return sim.dumpData()


def run_batch(pbf, solver, scenes, steps, waves=None):
    with pbf.Batch(solver, *capacity(scenes)) as b:
        ids = [b.add_scene(s.params, s.particles) for s in scenes]
        for i, w in (waves or {}).items():
            b.set_wave(ids[i], w)
        b.step(steps)
        return [b.dump_scene(i) for i in ids]


def assert_same(got, want, what):
    for g, w, nm in zip(got, want, ("positions", "velocities")):
        assert g.shape == w.shape
        diff = np.flatnonzero((bits(g) != bits(w)).any(axis=1))
        assert diff.size == 0, f"{what}: {nm} differ at {diff.size} particles (first {diff[:5]})"


def test_batch_matches_plain_simulation_bitwise(pbf):
    scenes = plain_scenes(pbf)
    got = run_batch(pbf, scenes[0].params, scenes, 25)
    for s, g in zip(scenes, got):
        assert_same(g, run_plain(pbf, s, 25), f"scene {s.name}")


def test_batch_neighbour_stats_match_the_plain_simulations(pbf):
    """The batch's list statistics are those of its scenes stepped alone
    (largest count the largest of theirs, overflows their sum), also with a
    capacity small enough that some particles overflow; none before a step
    on the current layout."""
    scenes = plain_scenes(pbf)
    for cap in (128, 16):
        solver = scenes[0].params.copy()
        solver.max_neighbours = cap
        alone = []
        for s in scenes:
            p = s.params.copy()
            p.max_neighbours = cap
            p.grow_lists = 0
            with pbf.Simulation(p, s.particles) as sim:
                sim.init()
                sim.step(5)
                alone.append(sim.neighbour_stats())
        with pbf.Batch(solver, *capacity(scenes)) as b:
            for s in scenes:
                b.add_scene(s.params, s.particles)
            with pytest.raises(pbf.PbfError) as e:
                b.neighbour_stats()
            assert e.value.status == pbf.ERR_STATE
            b.step(0)  # applies the layout and captures the step, steps nothing
            with pytest.raises(pbf.PbfError) as e:
                b.neighbour_stats()
            assert e.value.status == pbf.ERR_STATE
            b.step(5)
            mx, over = b.neighbour_stats()
            b.set_tuning(b.tuning())  # a new launch shape keeps the lists
            assert b.neighbour_stats() == (mx, over)
        assert mx == max(m for m, _ in alone)
        assert over == sum(o for _, o in alone)
        assert (over > 0) == (cap == 16)


def test_mixed_sizes_alone_vs_mix_bitwise(pbf):
    scenes = pbf.scenes.mixed_batch(count=8, n_min=1000, n_max=30000, seed=7)
    solver = scenes[0].params
    mix = run_batch(pbf, solver, scenes, 20)
    for s, g in zip(scenes, mix):
        alone = run_batch(pbf, solver, [s], 20)[0]
        assert_same(g, alone, f"scene {s.name} (n={s.n})")
        assert np.isfinite(g[0]).all()


def test_remove_and_add_between_steps(pbf):
    a, b, c, d = plain_scenes(pbf)
    e = pbf.scenes.dam_break((10, 10, 10), (0.8, 1.6, 0.8), seed=15, name="e")
    cap = capacity([a, b, c, d, e])
    with pbf.Batch(a.params, *cap) as bt:
        ids = {s.name: bt.add_scene(s.params, s.particles) for s in (a, b, c, d)}
        bt.step(10)
        bt.remove_scene(ids["b"])
        assert bt.info()[0] == 3
        ids["e"] = bt.add_scene(e.params, e.particles)
        bt.step(10)
        out = {nm: bt.dump_scene(i) for nm, i in ids.items() if nm != "b"}
        with pytest.raises(pbf.PbfError) as ex:
            bt.dump_scene(ids["b"])
        assert ex.value.status == pbf.ERR_NOT_FOUND
    for s in (a, c, d):
        assert_same(out[s.name], run_plain(pbf, s, 20), f"scene {s.name}")
    assert_same(out["e"], run_plain(pbf, e, 10), "scene e (added after 10 steps)")


def test_wave_is_per_scene(pbf):
    a, b = plain_scenes(pbf)[:2]
    got = run_batch(pbf, a.params, [a, b], 15, waves={0: 0.05})
    assert_same(got[0], run_plain(pbf, a, 15, wave=0.05), "scene a with wave")
    assert_same(got[1], run_plain(pbf, b, 15), "scene b without wave")


def test_batch_step_matches_fp64_oracle(pbf, oracle_mod):
    scenes = plain_scenes(pbf)
    got = run_batch(pbf, scenes[0].params, scenes, 1)
    for s, (gp, gv) in zip(scenes, got):
        pos, vel = pbf.state_from_particles(s.particles)
        prm = ge.paper_params_for_oracle(s.params)
        op, ov, _, _, _ = oracle_mod.paper_steps_f64(prm, pos.astype(np.float64), vel.astype(np.float64), 1)
        err = np.abs(gp[:, :3].astype(np.float64) - op[:, :3]).max()
        assert err <= POS_TOL_H * s.params.h, f"scene {s.name}: {err / s.params.h:.3e} h"


def test_capacity_is_enforced(pbf):
    a, _, c, _ = plain_scenes(pbf)
    with pbf.Batch(a.params, 2, a.n + c.n // 2, a.params.ncells + c.params.ncells) as bt:
        bt.add_scene(a.params, a.particles)
        with pytest.raises(pbf.PbfError) as ex:
            bt.add_scene(c.params, c.particles)
        assert ex.value.status == pbf.ERR_BUDGET
        bt.add_scene(c.params, c.particles[: c.n // 2])
        with pytest.raises(pbf.PbfError) as ex:
            bt.add_scene(c.params, c.particles[:1])
        assert ex.value.status == pbf.ERR_BUDGET
        bt.step(2)
        assert bt.info() == (2, a.n + c.n // 2, a.params.ncells + c.params.ncells)


def test_launch_count_is_independent_of_scene_count(pbf):
    scenes = plain_scenes(pbf)
    with pbf.Batch(scenes[0].params, *capacity(scenes)) as bt:
        bt.add_scene(scenes[0].params, scenes[0].particles)
        one = bt.launches_per_step()
        for s in scenes[1:]:
            bt.add_scene(s.params, s.particles)
        many = bt.launches_per_step()
    # only the number of radix passes may grow with the key range
    assert many - one <= 1
    assert one <= 20
