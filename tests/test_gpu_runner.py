"""The headless runner (pbf_run, pbf::Runner) with the part_out / vtk_out
snapshot keys: files appear at the stated steps, and a .in snapshot is the
simulation's state at that step bit for bit (the .in text round-trips
float32 exactly)."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_runner_snapshots(pbf, tmp_path):
    sc = pbf.scenes.dam_break((6, 6, 6), (0.8, 0.8, 0.8), seed=61)
    p = sc.params.copy()
    p.part_input_file = b"s.in"
    p.time_end = np.float32(10.5 * p.time_step_length)
    p.part_out_freq = 4
    p.part_out_name_base = str(tmp_path / "snap_").encode()
    p.vtk_out_freq = 8
    p.vtk_out_name_base = str(tmp_path / "frame_").encode()
    pbf.write_particles(tmp_path / "s.in", sc.particles)
    pbf.write_config(tmp_path / "s.par", p)
    runner = pbf.PKG_DIR / "pbf_run"
    out = subprocess.run([str(runner), str(tmp_path / "s.par")], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    assert "mean:" in out.stdout
    assert (tmp_path / "snap_00001.in").exists() and (tmp_path / "snap_00002.in").exists()
    assert (tmp_path / "frame_00001.vtk").exists()
    assert not (tmp_path / "snap_00003.in").exists()
    got = pbf.read_particles(tmp_path / "snap_00002.in")
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        sim.step(8)
        pos, vel = sim.dumpData()
    assert np.array_equal(got["x"], pos[:, :3]) and np.array_equal(got["v"], vel[:, :3])
    assert np.array_equal(got["m"], vel[:, 3])
    raw = (tmp_path / "frame_00001.vtk").read_bytes()
    assert raw.startswith(b"# vtk DataFile Version 3.0") and b"POINTS %d float" % sc.n in raw
