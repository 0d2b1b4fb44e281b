"""The C-ABI library on the host (no GPU calls): it loads, exports every
function include/pbf.h declares, and its host-only entry points (scenario
readers, generator, parameter validation) behave like the reference's."""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions() -> list[str]:
    text = (ROOT / "include" / "pbf.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pbf_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(pbf):
    lib = C.CDLL(str(pbf.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares every one of them
    bound = set(pbf.exported_symbols())
    assert set(names) <= bound, set(names) - bound


def test_abi_version_and_status_strings(pbf):
    L = pbf.lib()
    assert L.pbf_abi_version() == 1
    for s in range(9):
        assert L.pbf_status_string(s)
    assert L.pbf_status_string(99) == b"unknown status"


def test_params_defaults(pbf):
    p = pbf.default_params()
    assert p.mode == pbf.MODE_PAPER
    assert p.solver_iterations == 4
    assert p.relax_eps == pytest.approx(600.0)
    assert p.scorr_k == pytest.approx(0.1) and p.scorr_n == 4 and p.scorr_dq == pytest.approx(0.2)
    assert p.xsph_c == pytest.approx(0.01) and p.vort_eps == pytest.approx(0.0005)
    assert p.gravity_y == pytest.approx(-9.81)
    assert p.max_neighbours == 128


PAR_TEXT = """part_input_file       two.in
time_end              100.0
timestep_length       0.005
x_min                 0
y_min                 0
z_min                 0
x_max                 1
y_max                 1
z_max                 1
x_n                   100
y_n                   100
z_n                   100
restdensity           998200.0
part_out_freq         7
part_out_name_base    out
vtk_out_freq          3
vtk_out_name_base     vtk
cl_workgroup_1dsize   64
some_unknown_key      5
mode                  ref_compat
solver_iterations     6
relax_eps             1234.5
"""


def test_read_config(pbf, tmp_path, capfd):
    path = tmp_path / "two.par"
    path.write_text(PAR_TEXT)
    p = pbf.read_config(path)
    assert p.part_input_file == b"two.in"
    assert p.time_end == 100.0 and p.time_step_length == np.float32(0.005)
    assert (p.x_max, p.y_max, p.z_max) == (1.0, 1.0, 1.0)
    assert (p.x_n, p.y_n, p.z_n) == (100.0, 100.0, 100.0)
    assert p.rest_density == np.float32(998200.0)
    assert p.part_out_freq == 7 and p.part_out_name_base == b"out"
    assert p.vtk_out_freq == 3 and p.vtk_out_name_base == b"vtk"
    assert p.cl_workgroup_1dsize == 64
    assert p.mode == pbf.MODE_REF_COMPAT and p.solver_iterations == 6
    assert p.relax_eps == np.float32(1234.5)
    err = capfd.readouterr().err
    assert "Unknown parameter some_unknown_key" in err


def test_read_config_errors(pbf, tmp_path):
    with pytest.raises(pbf.PbfError) as e:
        pbf.read_config(tmp_path / "missing.par")
    assert e.value.status == pbf.ERR_IO
    bad = tmp_path / "bad.par"
    bad.write_text("x_n notanumber\n")
    with pytest.raises(pbf.PbfError):
        pbf.read_config(bad)


def test_read_particles(pbf, tmp_path, golden):
    pos0, vel0 = golden["dam/pos0"], golden["dam/vel0"]
    lines = [str(pos0.shape[0])]
    for p, v in zip(pos0, vel0):
        lines.append(" ".join(repr(float(t)) for t in [v[3], *p[:3], *v[:3]]))
    path = tmp_path / "dam.in"
    path.write_text("\n".join(lines) + "\n")
    ps = pbf.read_particles(path)
    assert ps.shape[0] == pos0.shape[0]
    assert np.array_equal(ps["x"], pos0[:, :3])
    assert np.array_equal(ps["v"], vel0[:, :3])
    assert np.array_equal(ps["m"], vel0[:, 3])
    # a malformed line ends the read with what was parsed so far
    bad = tmp_path / "bad.in"
    bad.write_text("3\n1 0 0 0 0 0 0\n1 0 0 zz 0 0 0\n1 0 0 0 0 0 0\n")
    assert pbf.read_particles(bad).shape[0] == 1
    with pytest.raises(pbf.PbfError):
        pbf.read_particles(tmp_path / "missing.in")


def test_data_path(pbf):
    assert pbf.data_path("/x", "scenario", "dam.par") == "/x/data/scenarios/dam.par"
    assert pbf.data_path("/x", "kernel", "a.cl") == "/x/data/kernels/a.cl"
    with pytest.raises(pbf.PbfError):
        pbf.data_path("/x", "nope", "a")


def _splitmix64(state):
    mask = (1 << 64) - 1
    state = (state + 0x9E3779B97F4A7C15) & mask
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
    return state, z ^ (z >> 31)


def test_generate_block_matches_spec(pbf):
    ps = pbf.generate_block((0.1, 0.2, 0.3), 3, 4, 5, 0.05, 0.0005, 0.125, 99)
    assert ps.shape == (60,)
    state = 99
    q = 0
    for ix in range(3):
        for iy in range(4):
            for iz in range(5):
                for a, idx in enumerate((ix, iy, iz)):
                    state, z = _splitmix64(state)
                    u = (z >> 11) * (1.0 / 9007199254740992.0)
                    origin = np.float64(np.float32((0.1, 0.2, 0.3)[a]))
                    spacing = np.float64(np.float32(0.05))
                    jitter = np.float64(np.float32(0.0005))
                    want = np.float32(origin + idx * spacing + (2 * u - 1) * jitter)
                    assert ps["x"][q, a] == want
                q += 1
    assert (ps["m"] == np.float32(0.125)).all() and (ps["v"] == 0).all()
    again = pbf.generate_block((0.1, 0.2, 0.3), 3, 4, 5, 0.05, 0.0005, 0.125, 99)
    assert np.array_equal(ps, again)


def test_create_validation(pbf):
    sc = pbf.scenes.config_small()
    ok = sc.params
    cases = []
    p = ok.copy(); p.x_n = 0; cases.append(p)
    p = ok.copy(); p.x_n = 2.5; cases.append(p)
    p = ok.copy(); p.time_step_length = 0; cases.append(p)
    p = ok.copy(); p.rest_density = -1; cases.append(p)
    p = ok.copy(); p.solver_iterations = 0; cases.append(p)
    p = ok.copy(); p.mode = 7; cases.append(p)
    p = ok.copy(); p.y_n = 32; cases.append(p)  # paper mode: y cells shorter than h
    p = ok.copy(); p.max_neighbours = 0; cases.append(p)
    for bad in cases:
        with pytest.raises(pbf.PbfError) as e:
            pbf.Simulation(bad, sc.particles)
        assert e.value.status == pbf.ERR_INVALID
    with pytest.raises(pbf.PbfError):
        pbf.Simulation(ok, sc.particles[:0])
    # ref-compat accepts any grid the reference accepts
    p = ok.copy(); p.mode = pbf.MODE_REF_COMPAT; p.y_n = 32
    s = pbf.Simulation(p, sc.particles)
    # calls before init report a state error, not a crash
    with pytest.raises(pbf.PbfError) as e:
        s.step(1, sync=False)
    assert e.value.status == pbf.ERR_STATE
    with pytest.raises(pbf.PbfError) as e:
        s.neighbour_stats()
    assert e.value.status == pbf.ERR_STATE
    s.close()


def test_batch_host_checks(pbf):
    """Batch arguments rejected before any device work."""
    sc = pbf.scenes.config_small()
    ref = sc.params.copy()
    ref.mode = pbf.MODE_REF_COMPAT
    for args in ((ref, 4, 1000, 1000), (sc.params, 0, 1000, 1000), (sc.params, 70000, 1000, 1000),
                 (sc.params, 4, 0, 1000), (sc.params, 4, 1000, 0)):
        with pytest.raises(pbf.PbfError) as e:
            pbf.Batch(*args)
        assert e.value.status == pbf.ERR_INVALID
    small = pbf.Batch.device_bytes(sc.params, 4, 1 << 16, 1 << 16)
    big = pbf.Batch.device_bytes(sc.params, 256, 16 << 20, 16 << 20)
    assert 0 < small < big
    # a 16M-particle batch stays well inside one GB300
    assert big < 16 * (1 << 30)
    # server arguments and budgets that hold no batch
    for args, kw in (((sc.params, 1 << 30), {"max_scenes": 0}), ((sc.params, 1 << 30), {"max_chunk": 0}),
                     ((sc.params, 1 << 30), {"cells_per_particle": 0.5}), ((ref, 1 << 30), {})):
        with pytest.raises(pbf.PbfError) as e:
            pbf.Server(*args, **kw)
        assert e.value.status == pbf.ERR_INVALID
    with pytest.raises(pbf.PbfError) as e:
        pbf.Server(sc.params, 1 << 16)
    assert e.value.status == pbf.ERR_BUDGET


def test_scenes_shapes(pbf):
    s1 = pbf.scenes.config_small()
    assert s1.n == 32768 and s1.params.ncells == 16 * 16 * 32
    s2 = pbf.scenes.config_1m()
    assert s2.n == 1048576 and s2.params.ncells == 64 ** 3
    # blocks sit inside the paper-mode walls
    m = s2.params.wall_margin
    x = s2.particles["x"]
    assert x.min() >= -1e-3 + m and x[:, 0].max() <= 6.4 - m + 1e-3
    b = pbf.scenes.mixed_batch(16)
    assert len(b) == 16 and all(4096 * 0.9 <= s.n <= 262144 * 1.1 for s in b)


def test_ppm_writer(pbf, tmp_path):
    img = np.zeros((3, 4, 3), np.uint8)
    img[0, 0] = (255, 0, 0)
    p = tmp_path / "x.ppm"
    pbf.write_ppm(p, img)
    data = p.read_bytes()
    assert data.startswith(b"P6\n4 3\n255\n") and len(data) == len(b"P6\n4 3\n255\n") + 36


def test_render_restatement_single_particle(pbf):
    """The renderer's oracle: one particle at the box centre seen by the
    reference's initial camera is a disc at the image centre, (|v|, |v|, 1)
    at its middle (normal towards the camera), on the 0.05 grey background."""
    from oracle import render as oracle_render

    sc = pbf.scenes.dam_break((2, 2, 2), (0.8, 0.8, 0.8), seed=1)
    cam = pbf.default_camera(sc.params)
    assert cam.theta_deg == 20.0 and cam.fovy_deg == 45.0 and abs(cam.distance + 1.6) < 1e-6
    cam.max_point_size = 256.0
    pos = np.array([[0.4, 0.4, 0.4, 0.5]], np.float32)
    img = oracle_render.render(pos, sc.params, cam, 400, 300)
    assert tuple(img[0, 0]) == (13, 13, 13)
    c = img[150, 200].astype(int)
    assert abs(c[0] - 128) <= 2 and c[0] == c[1] and c[2] == 255
    covered = (img != 13).any(axis=2)  # unlit parts of the sphere are black, not background
    ys, xs = np.nonzero(covered)
    assert abs(xs.mean() - 199.5) < 1.5 and abs(ys.mean() - 149.5) < 1.5
    # 200 / w pixels across, w = the distance along the view axis (1.6 m)
    assert abs((xs.max() - xs.min() + 1) - 200 / 1.6) <= 2


def test_selftest_argument_checks(pbf):
    flag = C.c_uint32()
    assert pbf.lib().pbf_selftest_bounded_wait(0, C.byref(flag)) == pbf.ERR_INVALID
    assert pbf.lib().pbf_selftest_bounded_wait(1 << 27, C.byref(flag)) == pbf.ERR_INVALID
    assert pbf.lib().pbf_selftest_bounded_wait(100, None) == pbf.ERR_INVALID


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "pbf.h"

/* every entry point pbf.h declares, referenced so the linker resolves each */
static void *const entry_points[] = {
%s
};

int main(void) {
  pbf_params p;
  pbf_params_default(&p);
  if (pbf_abi_version() != 1) return 1;
  if (strcmp(pbf_status_string(PBF_ERR_INVALID), "invalid argument") != 0) return 2;
  printf("abi %%d entry points %%zu h %%g\n", pbf_abi_version(),
         sizeof entry_points / sizeof entry_points[0], (double)((p.x_max - p.x_min) / p.x_n));
  return 0;
}
"""


def test_header_is_c_and_every_entry_point_links(pbf, tmp_path):
    """A C11 caller (gcc -Wall -Wextra -Werror) includes pbf.h, takes the
    address of every function it declares, links against the library and
    runs its host-only entry points -- the boundary as a C program sees it."""
    import shutil
    import subprocess

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    names = declared_functions()
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER % ",\n".join(f"    (void *){n}" for n in names))
    exe = tmp_path / "caller"
    lib_dir = pbf.LIB_PATH.parent
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-Wno-pedantic", f"-I{ROOT / 'include'}",
           str(src), f"-L{lib_dir}", f"-l:{pbf.LIB_PATH.name}", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert f"entry points {len(names)}" in out.stdout and "h 0.1" in out.stdout
