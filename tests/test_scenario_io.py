"""Scenario I/O on the host: .in text and binary particle files, .par
writing, the tools/gen_grid.py scenario pair, VTK output."""
from __future__ import annotations

import numpy as np


def test_particle_text_round_trip(pbf, tmp_path):
    ps = pbf.generate_block((0.1, 0.2, 0.3), 5, 4, 3, 0.05, 0.0005, 0.125, 7)
    ps["v"] = np.random.default_rng(1).normal(size=(60, 3)).astype(np.float32)
    pbf.write_particles(tmp_path / "a.in", ps)
    back = pbf.read_particles(tmp_path / "a.in")
    for f in ("m", "x", "v"):
        assert np.array_equal(back[f], ps[f]), f
    first = (tmp_path / "a.in").read_text().splitlines()[:2]
    assert first[0] == "60" and len(first[1].split()) == 7


def test_particle_binary_round_trip(pbf, tmp_path):
    ps = pbf.generate_block((0.0, 0.0, 0.0), 10, 10, 10, 0.05, 0.001, 0.125, 9)
    pbf.write_particles(tmp_path / "a.pbin", ps, binary=True)
    raw = (tmp_path / "a.pbin").read_bytes()
    assert raw[:4] == b"PBFB" and len(raw) == 16 + 1000 * 40
    back = pbf.read_particles(tmp_path / "a.pbin")
    assert np.array_equal(back, ps)


def test_config_round_trip(pbf, tmp_path):
    p = pbf.scenes.config_small().params.copy()
    p.part_input_file = b"x.in"
    p.part_out_freq = 5
    p.part_out_name_base = b"snap_"
    p.vtk_out_freq = 10
    p.mode = pbf.MODE_REF_COMPAT
    pbf.write_config(tmp_path / "c.par", p)
    q = pbf.read_config(tmp_path / "c.par")
    for name, _ in pbf.Params._fields_:
        a, b = getattr(p, name), getattr(q, name)
        if name == "vtk_out_name_base" and not a:
            assert b == b"vtk"
            continue
        assert a == b, name


def test_gen_grid_pair(pbf, tmp_path):
    pin, ppar = pbf.scenes.gen_grid(tmp_path)
    ps = pbf.read_particles(pin)
    assert ps.shape[0] == 21 ** 3
    assert (ps["m"] == 1).all() and (ps["v"] == 0).all()
    assert tuple(ps["x"][0]) == (10.0, 10.0, 10.0) and tuple(ps["x"][-1]) == (20.0, 20.0, 20.0)
    assert tuple(ps["x"][1]) == (10.0, 10.0, 10.5)  # z innermost, x outermost
    p = pbf.read_config(ppar)
    assert p.part_input_file == b"dam_coarse.in"
    assert (p.x_n, p.x_max, p.time_step_length) == (30.0, 30.0, np.float32(0.01))
    assert p.rest_density == np.float32(21 ** 3 / 1000.0)


def test_vtk_layout(pbf, tmp_path):
    pos = np.zeros((3, 4), np.float32)
    pos[:, 0] = [1, 2, 3]
    pos[:, 3] = [0.5, 1.5, 2.5]
    vel = np.ones((3, 4), np.float32)
    pbf.write_vtk(tmp_path / "a.vtk", pos, vel)
    raw = (tmp_path / "a.vtk").read_bytes()
    assert raw.startswith(b"# vtk DataFile Version 3.0\n")
    assert b"POINTS 3 float\n" in raw and b"VERTICES 3 6\n" in raw and b"SCALARS speed float 1" in raw
    i = raw.index(b"POINTS 3 float\n") + len(b"POINTS 3 float\n")
    assert np.frombuffer(raw[i:i + 36], ">f4").reshape(3, 3)[:, 0].tolist() == [1, 2, 3]
