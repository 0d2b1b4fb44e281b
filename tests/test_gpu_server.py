"""Served scenes (pbf_server_*): requests admitted while others run.

Equality statement (checked below): the final state of every request is
BIT-IDENTICAL to the same scene stepped alone for the same number of steps
through the plain simulation, whatever requests it shared the device with,
when they were admitted, and how the loop chunked the steps.  Requests
arrive between turns of the loop, so later ones join a batch that is already
running.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def exact_h_scenes(pbf):
    """Scenes whose cell length is exactly h = 0.1 (extents 0.1 x 2^k)."""
    dam = pbf.scenes.dam_break
    return [dam((12, 10, 14), (1.6, 1.6, 1.6), seed=21, name="a"),
            dam((20, 16, 8), (1.6, 1.6, 0.8), seed=22, name="b"),
            dam((6, 6, 6), (0.8, 0.8, 0.8), seed=23, name="c"),
            dam((24, 12, 12), (3.2, 1.6, 1.6), seed=24, name="d"),
            dam((10, 10, 10), (0.8, 1.6, 0.8), seed=25, name="e"),
            dam((16, 8, 16), (1.6, 0.8, 1.6), seed=26, name="f")]


def alone(pbf, scene, steps):
    with pbf.Simulation(scene.params, scene.particles) as sim:
        sim.init()
        sim.step(steps)
        return sim.dumpData()


def assert_same(got, want, what):
    for g, w, nm in zip(got, want, ("positions", "velocities")):
        diff = np.flatnonzero((bits(g) != bits(w)).any(axis=1))
        assert diff.size == 0, f"{what}: {nm} differ at {diff.size} particles"


def test_requests_alone_vs_mix_bitwise(pbf):
    scenes = exact_h_scenes(pbf)
    steps = [23, 17, 31, 12, 19, 5]
    with pbf.Server(scenes[0].params, 512 << 20, max_scenes=16, max_chunk=4) as srv:
        rids = {}
        for s, k in zip(scenes[:3], steps[:3]):
            rids[s.name] = srv.submit(s.params, s.particles, k)
        # a few turns with the first requests on the device, then more arrive
        for _ in range(3):
            srv.poll(wait=True)
        assert srv.stats()["active"] == 3
        for s, k in zip(scenes[3:], steps[3:]):
            rids[s.name] = srv.submit(s.params, s.particles, k)
        done = srv.run_until_idle()
        st = srv.stats()
        assert st["completed"] == 6 and st["active"] == 0 and st["queued"] == 0
        results = {nm: srv.result(r) for nm, r in rids.items()}
    assert len(done) >= 3
    for s, k in zip(scenes, steps):
        assert_same(results[s.name], alone(pbf, s, k), f"request {s.name} ({k} steps)")


def test_admission_respects_budget(pbf):
    scenes = exact_h_scenes(pbf)
    big = max(s.n for s in scenes)
    # a budget that holds about two of the scenes at a time
    solver = scenes[0].params
    budget = pbf.Batch.device_bytes(solver, 4, 2 * big + 64, 4 * (2 * big + 64))
    with pbf.Server(solver, budget, max_scenes=4, cells_per_particle=4.0, max_chunk=8) as srv:
        cap = srv.stats()
        assert cap["device_bytes"] <= budget
        rids = [srv.submit(s.params, s.particles, 9) for s in scenes]
        peak = 0
        busy = True
        while busy:
            _, busy = srv.poll(wait=True)
            st = srv.stats()
            assert st["active_particles"] <= cap["max_particles"]
            assert st["active_cells"] <= cap["max_cells"]
            peak = max(peak, st["active"])
        assert 1 <= peak < len(scenes)
        for s, r in zip(scenes, rids):
            assert_same(srv.result(r), alone(pbf, s, 9), f"request {s.name}")


def test_request_states_and_errors(pbf):
    a, _, c = exact_h_scenes(pbf)[:3]
    with pbf.Server(a.params, 256 << 20, max_scenes=8) as srv:
        big = pbf.scenes.dam_break((128, 128, 64), (6.4, 6.4, 6.4), seed=1)
        st = srv.stats()
        if big.n > st["max_particles"]:
            with pytest.raises(pbf.PbfError) as ex:
                srv.submit(big.params, big.particles, 10)
            assert ex.value.status == pbf.ERR_BUDGET
        r = srv.submit(c.params, c.particles, 40)
        assert srv.info(r)[0] == pbf.REQ_QUEUED
        srv.poll(wait=True)
        assert srv.info(r)[0] == pbf.REQ_ACTIVE
        with pytest.raises(pbf.PbfError) as ex:
            srv.result(r)
        assert ex.value.status == pbf.ERR_STATE
        srv.run_until_idle()
        state, n, k = srv.info(r)
        assert (state, n, k) == (pbf.REQ_DONE, c.n, 40)
        pos, _ = srv.result(r)
        assert np.isfinite(pos).all()
        with pytest.raises(pbf.PbfError) as ex:
            srv.result(r)
        assert ex.value.status == pbf.ERR_NOT_FOUND
        st = srv.stats()
        assert st["batch_steps"] == 40 and st["particle_steps"] == 40 * c.n
