"""The oracle itself (CPU): pinned against the reference's own kernels.

* The float REF_COMPAT restatement must equal, bit for bit, the reference's
  kernels compiled from their .cl sources -- live where the reference tree is
  present, and through the committed golden vectors everywhere.
* A pure-Python double-precision restatement of the reference equations for
  tiny scenes (brute-force neighbours) checks both independently.
* The sort-path intent (hash, stable permutation, inclusive ranges) must
  reproduce the cell membership of the reference's linked cell lists.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import golden_scenarios, oracle_config


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


# ------------------------------------------------------------------ pinning
def test_restatement_matches_golden_bit_for_bit(golden, oracle_mod):
    for name in golden_scenarios(golden):
        cfg = oracle_config(oracle_mod, golden[f"{name}/config"])
        pos0, vel0 = golden[f"{name}/pos0"], golden[f"{name}/vel0"]
        for k in golden[f"{name}/steps"]:
            pos, vel, pred, sc = oracle_mod.refcompat_steps_f32(cfg, pos0, vel0, int(k),
                                                                want_predicted=True, want_scaling=True)
            assert np.array_equal(bits(pos), bits(golden[f"{name}/k{k}/pos"])), (name, k)
            assert np.array_equal(bits(vel), bits(golden[f"{name}/k{k}/vel"])), (name, k)
            assert np.array_equal(bits(pred), bits(golden[f"{name}/k{k}/pred"])), (name, k)
            assert np.array_equal(bits(sc), bits(golden[f"{name}/k{k}/scaling"])), (name, k)


def test_restatement_matches_live_reference(oracle_mod):
    if not oracle_mod.reference_available():
        pytest.skip("the reference's kernels are not buildable on this host")
    from oracle.build import REFERENCE_SCENARIOS as scen

    if not scen.is_dir():
        pytest.skip("reference scenarios not present")
    for name, steps in [("dam2", 3), ("drop", 3), ("dam_coarse", 3), ("dam_miles", 10), ("box_big", 10)]:
        cfg = oracle_mod.read_par(scen / f"{name}.par")
        pos0, vel0 = oracle_mod.read_in(scen / f"{name}.in")
        a = oracle_mod.reference_steps(cfg, pos0, vel0, steps, threads=4)
        b = oracle_mod.refcompat_steps_f32(cfg, pos0, vel0, steps, threads=4, want_predicted=True,
                                           want_scaling=True)
        for x, y in zip(a[:4], b):
            assert np.array_equal(bits(x), bits(y)), name


def test_constants_follow_main_cpp(oracle_mod, golden):
    # h = 0.1: the literals src/main.cpp prints with 6 significant digits.
    cfg = oracle_mod.Config(0, 1.6, 0, 1.6, 0, 3.2, 16, 16, 32, 1 / 120, 8000)
    k = oracle_mod.ref_constants(cfg)
    assert k[14] == np.float32(0.100000)
    assert k[16] == np.float32(1.56668e09)
    assert k[17] == np.float32(1.43239e07)
    assert k[12] == np.float32(0.00833333)
    if oracle_mod.reference_available():
        for name in golden_scenarios(golden):
            c = oracle_config(oracle_mod, golden[f"{name}/config"])
            assert np.array_equal(oracle_mod.ref_constants(c), oracle_mod.reference_constants(c))


# ------------------------------------------------- independent restatement
def _python_ref_step(k, pos, vel, iters=4):
    """Pure-Python double restatement of one reference step (brute-force
    neighbour search; equal to the 27-cell scan when cells are >= h)."""
    (mn, mx, dt, rd, h, h2, poly6, spiky) = k
    n = len(pos)
    x = [list(map(float, p[:3])) for p in pos]
    v = [list(map(float, q[:3])) for q in vel]
    g = float(np.float32(-9.81))  # predict_positions.cl:8 float literal
    c = float(np.float32(0.01))  # apply_vorticity_and_viscosity.cl:103
    for i in range(n):
        v[i][1] += dt * g
    p = [[x[i][a] + dt * v[i][a] for a in range(3)] for i in range(n)]
    rho = [0.0] * n
    for _ in range(iters):
        lam = [0.0] * n
        for i in range(n):
            dens, gsum, gv = 0.0, 0.0, [0.0, 0.0, 0.0]
            for j in range(n):
                if i == j:
                    continue
                r = [p[i][a] - p[j][a] for a in range(3)]
                r2 = sum(c * c for c in r)
                if 0 < r2 < h2:
                    rl = math.sqrt(r2)
                    g = [c / rl * spiky * (h - rl) ** 2 for c in r]
                    dens += poly6 * (h2 - r2) ** 3
                    gsum += math.sqrt(sum(c * c for c in g))
                    gv = [gv[a] + g[a] for a in range(3)]
            gsum += math.sqrt(sum(c * c for c in gv))
            rho[i] = dens
            lam[i] = -(dens / rd - 1.0) / (gsum * gsum / (rd * rd) + 1e4)
        newp = []
        for i in range(n):
            s = [0.0, 0.0, 0.0]
            for j in range(n):
                if i == j:
                    continue
                r = [p[i][a] - p[j][a] for a in range(3)]
                r2 = sum(c * c for c in r)
                if 0 < r2 < h2:
                    rl = math.sqrt(r2)
                    s = [s[a] - (lam[i] + lam[j]) * r[a] / rl * spiky * (h - rl) ** 2 for a in range(3)]
            f = [p[i][a] + s[a] / rd for a in range(3)]
            for a in range(3):
                if f[a] - h < mn[a]:
                    f[a] = mn[a] + h
                elif f[a] + h > mx[a]:
                    f[a] = mx[a] - h
            newp.append(f)
        p = newp
    v = [[(p[i][a] - x[i][a]) / dt for a in range(3)] for i in range(n)]
    dv = []
    for i in range(n):
        s = [0.0, 0.0, 0.0]
        for j in range(n):
            if i == j:
                continue
            r = [p[i][a] - p[j][a] for a in range(3)]
            r2 = sum(c * c for c in r)
            if 0 < r2 < h2:
                w = poly6 * (h2 - r2) ** 3 / rho[j]
                s = [s[a] + (v[j][a] - v[i][a]) * w for a in range(3)]
        dv.append([c * q for q in s])
    v = [[v[i][a] + dv[i][a] for a in range(3)] for i in range(n)]
    return np.array(p), np.array(v), np.array(rho)


@pytest.mark.parametrize("name", ["two", "two_updown", "box_small", "27"])
def test_python_restatement_agrees(golden, oracle_mod, name):
    cfg = oracle_config(oracle_mod, golden[f"{name}/config"])
    k18 = oracle_mod.ref_constants(cfg).astype(np.float64)
    k = (k18[[0, 2, 4]], k18[[1, 3, 5]], k18[12], k18[13], k18[14], k18[15], k18[16], k18[17])
    pos0, vel0 = golden[f"{name}/pos0"], golden[f"{name}/vel0"]
    p, v, rho = _python_ref_step(k, pos0, vel0)
    opos, ovel = oracle_mod.refcompat_steps_f64(cfg, pos0, vel0, 1)
    scale = max(1.0, np.abs(opos[:, :3]).max())
    assert np.abs(p - opos[:, :3]).max() <= 1e-12 * scale
    assert np.abs(v - ovel[:, :3]).max() <= 1e-9 * max(1.0, np.abs(ovel[:, :3]).max())
    # float run of the reference kernels stays close to the double result
    g = golden[f"{name}/k1/pos"]
    assert np.abs(g[:, :3] - p).max() <= 2e-6 * scale


def test_two_particle_lambda_closed_form(golden, oracle_mod):
    """two.in: two particles 0.00423 apart on x with h = 0.01.  The first
    lambda of either particle has a closed form."""
    cfg = oracle_config(oracle_mod, golden["two/config"])
    k18 = oracle_mod.ref_constants(cfg).astype(np.float64)
    dt, rd, h, h2, poly6, spiky = k18[12:18]
    pos0 = golden["two/pos0"].astype(np.float64)
    r = abs(pos0[0, 0] - pos0[1, 0])
    dens = poly6 * (h2 - r * r) ** 3
    grad = spiky * (h - r) ** 2
    lam = -(dens / rd - 1.0) / ((2 * grad) ** 2 / rd ** 2 + 1e4)
    # One reference step with one iteration only: use the python restatement.
    kk = (k18[[0, 2, 4]], k18[[1, 3, 5]], dt, rd, h, h2, poly6, spiky)
    p, _, rho = _python_ref_step(kk, golden["two/pos0"], golden["two/vel0"], iters=1)
    assert rho[0] == pytest.approx(dens, rel=1e-12)
    dp = -2 * lam * grad / rd  # particle 0 sits at larger x: pulled toward -x
    assert p[0, 0] - (pos0[0, 0]) == pytest.approx(dp, rel=1e-9)


# ----------------------------------------------------------- sort intent
def test_hash_matches_reference_cell_lists(golden, oracle_mod):
    for name in golden_scenarios(golden):
        cfg = oracle_config(oracle_mod, golden[f"{name}/config"])
        for k in golden[f"{name}/steps"]:
            # the lists of the last step were built from the predicted
            # positions right after prediction; rebuild them from the step
            # start state with the live kernels where available, otherwise
            # compare against the recorded lists via the restated hash of
            # the predicted positions of the first step.
            if int(k) != 1:
                continue
            pos0, vel0 = golden[f"{name}/pos0"], golden[f"{name}/vel0"]
            dt = oracle_mod.ref_constants(cfg)[12]
            v = vel0.copy()
            v[:, 1] = v[:, 1] + dt * np.float32(-9.81)
            pred = pos0.copy()
            pred[:, :3] = pos0[:, :3] + dt * v[:, :3]
            h = oracle_mod.cell_hash(cfg, pred)
            assert np.array_equal(h, golden[f"{name}/k1/cell"]), name


def test_stable_sort_and_ranges(oracle_mod):
    rng = np.random.default_rng(3)
    for n, c in [(1, 1), (17, 4), (1000, 64), (5000, 10)]:
        h = rng.integers(0, c, n).astype(np.uint32)
        sk, perm = oracle_mod.sort_cells(h)
        assert np.array_equal(perm, np.argsort(h, kind="stable"))
        assert np.array_equal(sk, h[perm])
        fl = oracle_mod.find_cells(sk, c)
        for cell in range(c):
            idx = np.nonzero(sk == cell)[0]
            if idx.size:
                assert tuple(fl[cell]) == (idx[0], idx[-1])
            else:
                assert tuple(fl[cell]) == (-1, -1)


def test_reference_list_order_is_descending(golden, oracle_mod):
    if not oracle_mod.reference_available():
        pytest.skip("the reference's kernels are not buildable on this host")
    cfg = oracle_config(oracle_mod, golden["dam/config"])
    pos0 = golden["dam/pos0"]
    cells, lst = oracle_mod.reference_build_cells(cfg, pos0)
    for members in oracle_mod.cells_from_lists(cells, lst).values():
        assert members == sorted(members, reverse=True)


# ------------------------------------------------------- paper-equation oracle
def test_paper_oracle_conserves_momentum_without_walls(oracle_mod):
    """With no wall contact and no gravity, every delta-p pass is a sum of
    antisymmetric pair terms, so the total displacement is zero."""
    rng = np.random.default_rng(5)
    n = 400
    pos = np.zeros((n, 4))
    pos[:, :3] = 2.0 + rng.uniform(0, 0.4, (n, 3))
    vel = np.zeros((n, 4))
    vel[:, 3] = 0.125
    prm = oracle_mod.PaperParams()
    prm.box_min[:] = [0, 0, 0]
    prm.box_max[:] = [4.4, 4.4, 4.4]
    prm.n_cells[:] = [44, 44, 44]
    prm.iterations = 4
    prm.dt, prm.rest_density, prm.h = 1 / 120, 8000.0, 0.1
    prm.relax_eps, prm.scorr_k, prm.scorr_dq, prm.scorr_n = 600.0, 0.1, 0.2, 4
    prm.xsph_c, prm.vort_eps, prm.gravity_y, prm.wall_margin = 0.01, 0.0005, 0.0, 0.025
    out, ovel, dens, lam, cnt = oracle_mod.paper_steps_f64(prm, pos, vel, 1)
    disp = out[:, :3] - pos[:, :3]
    assert np.abs(disp.sum(0)).max() < 1e-12 * n
    assert cnt.max() > 0 and np.isfinite(out).all()
    # XSPH and vorticity terms conserve momentum only approximately (1/rho_j
    # weights); velocities stay finite and small.
    assert np.abs(ovel[:, :3]).max() < 10.0


def test_oracle_scenes_match_the_library_generator(oracle_mod):
    """The oracle builds the benchmark scenes itself (so that the CPU run of
    the reference's kernels loads nothing of the product); its generator
    equals pbf_generate_block bit for bit."""
    import __graft_entry__ as ge

    pbf = ge.load_package()
    for dims, seed in [((3, 4, 5), 7), ((16, 8, 4), 0x5EED), ((1, 1, 1), 2**64 - 1)]:
        ps = pbf.scenes.block((0.025, 0.025, 0.025), dims, seed)
        want_pos, want_vel = pbf.state_from_particles(ps)
        pos, vel = oracle_mod.generate_block((0.025, 0.025, 0.025), dims, 0.05, 0.0005, 0.125, seed)
        assert np.array_equal(bits(pos), bits(want_pos)), dims
        assert np.array_equal(bits(vel), bits(want_vel)), dims
    for (cfg, pos, vel), sc in [(oracle_mod.scene_1m(), pbf.scenes.config_1m()),
                                (oracle_mod.scene_small(), pbf.scenes.config_small())]:
        want_pos, want_vel = pbf.state_from_particles(sc.particles)
        assert np.array_equal(bits(pos), bits(want_pos)), sc.name
        assert np.array_equal(bits(vel), bits(want_vel)), sc.name
        p = sc.params
        for f, g in [("x_min", "x_min"), ("x_max", "x_max"), ("y_max", "y_max"), ("z_max", "z_max"),
                     ("x_n", "x_n"), ("y_n", "y_n"), ("z_n", "z_n"),
                     ("timestep_length", "time_step_length"), ("rest_density", "rest_density")]:
            assert np.float32(getattr(cfg, f)) == np.float32(getattr(p, g)), (sc.name, f)
        # the CPU arm's paper parameters are the product's for the same scene
        a = oracle_mod.benchmark_paper_params(cfg)
        b = ge.paper_params_for_oracle(p)
        for f, _ in oracle_mod.PaperParams._fields_:
            if f != "pad_":
                assert list(np.atleast_1d(getattr(a, f))) == list(np.atleast_1d(getattr(b, f))), \
                    (sc.name, f)


def test_scorr_taken_in_units_of_h2(oracle_mod):
    """s_corr = -k h^2 (W(r)/W(dq h))^n, the reading the paper equations use:
    with k = 0.1 a resting 16^3 block settles (mean density within 2% of
    rest, speeds below 1 m/s after 20 steps), while the literal k = 0.1 m^2
    (k h^2 with k = 10 at h = 0.1) outweighs lambda and throws the block
    apart within the same 20 steps."""
    cfg, pos, vel = oracle_mod.dam_break_scene((16, 16, 16), (1.6, 1.6, 1.6))
    prm = oracle_mod.benchmark_paper_params(cfg)
    prm.gravity_y = 0.0  # at rest: only the constraint and s_corr act
    out, ovel, dens, *_ = oracle_mod.paper_steps_f64(prm, pos, vel, 20, threads=0)
    assert np.isfinite(out).all()
    assert np.abs(ovel[:, :3]).max() < 1.0
    interior = dens > 0.8 * prm.rest_density
    assert abs(dens[interior].mean() / prm.rest_density - 1.0) < 0.02
    literal = oracle_mod.benchmark_paper_params(cfg)
    literal.gravity_y = 0.0
    literal.scorr_k = 0.1 / (literal.h * literal.h)
    out2, ovel2, *_ = oracle_mod.paper_steps_f64(literal, pos, vel, 20, threads=0)
    speed2 = np.abs(ovel2[:, :3]).max() if np.isfinite(ovel2).all() else np.inf
    assert speed2 > 50.0, speed2
