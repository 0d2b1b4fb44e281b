"""Headless renderer (pbf_render) against the numpy restatement of the
reference's particle drawing (oracle/render.py).

Both evaluate every expression in IEEE binary32, one rounded operation at a
time, in the same order (the CUDA translation unit is compiled without
contraction), so the images must be equal pixel for pixel; the render is
also deterministic (two renders are byte-identical).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["dam_break", "moving", "close_camera"])
def test_render_matches_restatement(pbf, case):
    from oracle import render as oracle_render

    sc = pbf.scenes.dam_break((8, 8, 8), (0.8, 0.8, 0.8), seed=41)
    steps = {"dam_break": 20, "moving": 45, "close_camera": 20}[case]
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        sim.step(steps)
        cam = pbf.default_camera(sc.params)
        if case == "close_camera":  # large sprites, up to the size cap
            cam.distance = cam.distance * 0.3
            cam.phi_deg, cam.theta_deg = 30.0, 35.0
        img = sim.render(cam, 120, 90)
        again = sim.render(cam, 120, 90)
        pos, _ = sim.dumpData()
    assert np.array_equal(img, again)
    ref = oracle_render.render(pos, sc.params, cam, 120, 90)
    lit = (ref.astype(int).sum(axis=2) > 3 * 13).mean()
    assert lit > 0.02  # the fluid is in view
    same = (img == ref).all(axis=2)
    assert same.all(), f"{(~same).sum()} pixels differ"


def test_batch_scene_renders_like_the_plain_simulation(pbf):
    sc = pbf.scenes.dam_break((10, 8, 6), (1.6, 0.8, 0.8), seed=42)
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        sim.step(5)
        want = sim.render(None, 96, 64)
    with pbf.Batch(sc.params, 1, sc.n, sc.params.ncells) as b:
        sid = b.add_scene(sc.params, sc.particles)
        b.step(5)
        got = b.render_scene(sid, sc.params, None, 96, 64)
    assert np.array_equal(got, want)
