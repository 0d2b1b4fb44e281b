"""Neighbour-list capacity that follows the scene (pbf_list_capacity).

A dense block (spacing 0.045 m instead of 0.05 m with h = 0.1 m, 1.37 times
the number density the rest density implies, so ~45 neighbours per
particle) started with lists of 32 entries: the first step's sets overflow,
the lists grow before the second step is launched, and no particle
re-derives its set in any later step.  The capacity never changes a result
bit (a run with large fixed lists gives the same bits), and one step from
the final state matches the FP64 oracle within 1e-5 h.
"""
from __future__ import annotations

import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def dense_scene(pbf):
    box = (1.6, 1.6, 1.6)
    cells = tuple(int(round(b / pbf.scenes.H)) for b in box)
    p = pbf.scenes.base_params(box, cells)
    ps = pbf.generate_block((0.1, 0.1, 0.1), 20, 20, 20, 0.045, 0.00045, pbf.scenes.MASS, 51)
    return p, ps


@pytest.mark.parametrize("staged", [0, 1])
def test_lists_grow_before_the_second_step(pbf, oracle_mod, staged):
    p, ps = dense_scene(pbf)
    p.max_neighbours = 32
    steps = 8
    with pbf.Simulation(p, ps) as sim:
        sim.init()
        t = sim.tuning()
        t.staged = staged
        sim.set_tuning(t)
        over = []
        for _ in range(steps):
            sim.step(1)
            sim.sync()
            over.append(sim.neighbour_stats())
        cap, grows = sim.list_capacity()
        got = sim.dumpData()
    assert over[0][1] > 0, "the first step should overflow 32-entry lists"
    assert all(o == 0 for _, o in over[1:]), over
    assert grows >= 1 and cap >= max(m for m, _ in over)
    fixed = p.copy()
    fixed.max_neighbours = 512
    fixed.grow_lists = 0
    with pbf.Simulation(fixed, ps) as sim:
        sim.init()
        sim.step(steps)
        ref = sim.dumpData()
        assert sim.list_capacity() == (512, 0)
    for g, r in zip(got, ref):
        assert np.array_equal(bits(g), bits(r))
    # one more step from the final state against the FP64 oracle
    pos, vel = got
    with pbf.Simulation(p, ps) as sim:
        sim.init()
        sim.set_state(pos, vel)
        sim.step(1)
        gp, _ = sim.dumpData()
    prm = ge.paper_params_for_oracle(p)
    op, *_ = oracle_mod.paper_steps_f64(prm, pos.astype(np.float64), vel.astype(np.float64), 1)
    assert np.abs(gp[:, :3].astype(np.float64) - op[:, :3]).max() <= 1e-5 * p.h


def test_fixed_lists_stay_fixed(pbf):
    p, ps = dense_scene(pbf)
    p.max_neighbours = 32
    p.grow_lists = 0
    with pbf.Simulation(p, ps) as sim:
        sim.init()
        sim.step(1)
        assert sim.neighbour_stats()[1] > 0  # overflowing sets re-derived
        sim.step(2)
        sim.sync()
        assert sim.list_capacity() == (32, 0)
