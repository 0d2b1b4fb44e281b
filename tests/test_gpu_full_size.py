"""The full-size workloads (1,048,576 and 4,194,304 particles, paper
equations), where running the FP64 oracle over many steps is too slow,
through properties that do not depend on size:

  * two runs from the same state give the same bits (fixed summation order);
  * the scene run inside a batch gives the same bits as the plain simulation
    (its cell length is exactly the batch's h);
  * neighbour lists capped at 16 entries -- most particles then re-derive
    their sets from the cells in every pass -- give the same bits as the
    default capacity (same members, same order, same arithmetic);
  * every position stays finite and inside the walls;

and one step of the 1M scene (from its initial block and from its state
after 12 steps) and of the 4.2M scene against the FP64 oracle on all host
cores (<= 1e-5 h in position; the measured error is printed as a JSON
line), the 1M scene's density error over its 500 steps, and two steps of
the 1M scene in REF_COMPAT mode bit for bit against the reference's own
kernels.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu

STEPS = 12


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def run(pbf, params, particles, steps):
    with pbf.Simulation(params, particles) as sim:
        sim.init()
        sim.step(steps)
        return sim.dumpData()


def inside_walls(params, pos):
    m = params.wall_margin
    lo = np.array([params.x_min, params.y_min, params.z_min]) + m
    hi = np.array([params.x_max, params.y_max, params.z_max]) - m
    p = pos[:, :3]
    return bool(np.isfinite(pos).all() and (p >= lo - 1e-5).all() and (p <= hi + 1e-5).all())


def test_single_scene_1m(pbf):
    sc = pbf.scenes.config_1m()
    ref = run(pbf, sc.params, sc.particles, STEPS)
    assert inside_walls(sc.params, ref[0])
    again = run(pbf, sc.params, sc.particles, STEPS)
    capped = sc.params.copy()
    capped.max_neighbours = 16
    capped.grow_lists = 0
    small_lists = run(pbf, capped, sc.particles, STEPS)
    with pbf.Batch(sc.params, 1, sc.n, sc.params.ncells) as bt:
        sid = bt.add_scene(sc.params, sc.particles)
        bt.step(STEPS)
        batched = bt.dump_scene(sid)
    for got in (again, small_lists, batched):
        for x, y in zip(got, ref):
            assert np.array_equal(bits(x), bits(y))


def test_double_dam_break_4m(pbf):
    sc = pbf.scenes.config_4m()
    ref = run(pbf, sc.params, sc.particles, 6)
    assert inside_walls(sc.params, ref[0])
    again = run(pbf, sc.params, sc.particles, 6)
    for x, y in zip(again, ref):
        assert np.array_equal(bits(x), bits(y))


def test_single_scene_1m_step_vs_fp64_oracle(pbf, oracle_mod):
    sc = pbf.scenes.config_1m()
    h = sc.params.h
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        sim.step(STEPS)
        moving = sim.dumpData()
    prm = ge.paper_params_for_oracle(sc.params)
    for label, (pos, vel) in (("initial block", pbf.state_from_particles(sc.particles)),
                              (f"step {STEPS}", moving)):
        with pbf.Simulation(sc.params, sc.particles) as sim:
            sim.init()
            sim.set_state(pos, vel)
            sim.step(1)
            gp, gv = sim.dumpData()
        op, ov, *_ = oracle_mod.paper_steps_f64(prm, pos.astype(np.float64), vel.astype(np.float64), 1)
        perr = np.abs(gp[:, :3].astype(np.float64) - op[:, :3]).max()
        vmax = np.abs(ov[:, :3]).max()
        verr = np.abs(gv[:, :3].astype(np.float64) - ov[:, :3]).max()
        print(json.dumps({"fp64_step_error": {"scene": sc.name, "particles": sc.n, "from": label,
                                              "pos_max_h": perr / h, "vel_max": verr, "vmax": vmax}}))
        assert perr <= 1e-5 * h, f"position error {perr / h:.3e} h"
        assert verr <= 1e-3 + 1e-4 * vmax, f"velocity error {verr}"


def test_single_scene_1m_density_over_500_steps(pbf):
    """Density error of the 1M dam break over its 500 steps, sampled every 10
    steps from each step's last lambda pass.  The 6.4 m water column is
    deeper than the 32,768-particle scene's, and 4 iterations with
    relaxation 600 are soft, so the impact (steps 60-160) compresses more.
    Measured: worst mean compression 0.264, worst max 3.32 (one particle in
    the splash), worst interior mean |rho/rho0 - 1| 0.266, settled mean
    compression after step 400 0.015.  Stated bounds, ~30% above.  The
    same samples check the neighbour lists: no particle exceeds the default
    list capacity (128), so none re-derives its set in the passes."""
    sc = pbf.scenes.config_1m()
    rho0 = sc.params.rest_density
    stats = []
    nbr = []
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        for k in range(50):
            sim.step(10)
            nbr.append(sim.neighbour_stats())
            rho = sim.density() / rho0
            comp = np.maximum(rho - 1.0, 0.0)
            interior = rho >= 0.8
            stats.append((10 * (k + 1), float(comp.mean()), float(comp.max()),
                          float(np.abs(rho[interior] - 1.0).mean())))
        pos, _ = sim.dumpData()
    worst = [max(s[i] for s in stats) for i in (1, 2, 3)]
    late = max(s[1] for s in stats if s[0] > 400)
    print(json.dumps({"density_error_500_steps_1m": {"mean_compression": worst[0],
                                                     "max_compression": worst[1],
                                                     "mean_abs_interior": worst[2],
                                                     "settled_mean_compression": late},
                      "neighbour_lists": {"max_count": max(m for m, _ in nbr),
                                          "overflow": max(o for _, o in nbr)}}))
    assert inside_walls(sc.params, pos)
    assert worst[0] <= 0.35 and worst[1] <= 4.5 and worst[2] <= 0.35
    assert late <= 0.02
    assert max(o for _, o in nbr) == 0


def test_double_dam_break_4m_step_vs_fp64_oracle(pbf, oracle_mod):
    """One step of the 4.2M double dam break, from its state after 6 steps,
    against the FP64 oracle on all host cores (<= 1e-5 h in position)."""
    sc = pbf.scenes.config_4m()
    h = sc.params.h
    pos, vel = run(pbf, sc.params, sc.particles, 6)
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        sim.set_state(pos, vel)
        sim.step(1)
        gp, gv = sim.dumpData()
    prm = ge.paper_params_for_oracle(sc.params)
    op, ov, *_ = oracle_mod.paper_steps_f64(prm, pos.astype(np.float64), vel.astype(np.float64), 1)
    perr = np.abs(gp[:, :3].astype(np.float64) - op[:, :3]).max()
    vmax = np.abs(ov[:, :3]).max()
    verr = np.abs(gv[:, :3].astype(np.float64) - ov[:, :3]).max()
    print(json.dumps({"fp64_step_error": {"scene": sc.name, "particles": sc.n, "from": "step 6",
                                          "pos_max_h": perr / h, "vel_max": verr, "vmax": vmax}}))
    assert perr <= 1e-5 * h, f"position error {perr / h:.3e} h"
    assert verr <= 1e-3 + 1e-4 * vmax, f"velocity error {verr}"


def test_single_scene_1m_ref_compat_matches_reference_kernels(pbf, oracle_mod):
    """REF_COMPAT at the headline size: two steps of the 1M scene in the
    reference's equations, bit for bit against the reference's own kernels
    (compiled from their .cl sources; cell lists built by a sequential
    update_cells launch, as the GPU path visits them) on all host cores."""
    if not oracle_mod.reference_available():
        pytest.skip("the reference's kernels are not built on this host")
    sc = pbf.scenes.config_1m()
    p = sc.params.copy()
    p.mode = pbf.MODE_REF_COMPAT
    cfg = oracle_mod.Config(p.x_min, p.x_max, p.y_min, p.y_max, p.z_min, p.z_max, p.x_n, p.y_n,
                            p.z_n, p.time_step_length, p.rest_density)
    pos0, vel0 = pbf.state_from_particles(sc.particles)
    rp, rv, rpred, *_ = oracle_mod.reference_steps(cfg, pos0, vel0, 2)
    with pbf.Simulation(p, sc.particles) as sim:
        sim.init()
        sim.initCells()
        sim.step(2)
        gp, gv = sim.dumpData()
        gd = sim.density()
    assert np.array_equal(bits(gp), bits(rp))
    assert np.array_equal(bits(gv), bits(rv))
    assert np.array_equal(bits(gd), bits(rpred[:, 3]))


def test_benchmark_mix_alone_vs_mix(pbf):
    """The 256-scene batched benchmark mix (14.6M particles, N log-uniform
    4,096-262,144) for 5 steps: eight scenes across the size range, each run
    alone in a batch of one, give the same bits as in the mix."""
    scenes = pbf.scenes.mixed_batch(256)
    solver = scenes[0].params
    n_tot = sum(s.n for s in scenes)
    cells = sum(s.params.ncells for s in scenes)
    pick = np.argsort([s.n for s in scenes])[np.linspace(0, len(scenes) - 1, 8).astype(int)]
    with pbf.Batch(solver, len(scenes), n_tot, cells) as bt:
        ids = [bt.add_scene(s.params, s.particles) for s in scenes]
        bt.step(5)
        mixed = {int(i): bt.dump_scene(ids[i]) for i in pick}
    for i in pick:
        s = scenes[int(i)]
        with pbf.Batch(solver, 1, s.n, s.params.ncells) as one:
            sid = one.add_scene(s.params, s.particles)
            one.step(5)
            alone = one.dump_scene(sid)
        assert inside_walls(s.params, alone[0])
        for x, y in zip(alone, mixed[int(i)]):
            assert np.array_equal(bits(x), bits(y)), s.name


def test_served_stream_alone_vs_mix(pbf):
    """The first 24 requests of the served benchmark stream (N log-uniform
    8,192-524,288, 100-1000 steps) submitted two per turn of the request
    loop under a 16 GB budget: four requests across the size range give the
    same bits as their scene stepped alone in a batch of one."""
    reqs = pbf.scenes.request_stream(1.0)[:24]
    scenes = [r.scene() for r in reqs]
    solver = scenes[0].params
    pick = [int(i) for i in np.argsort([r.n for r in reqs])[np.linspace(0, len(reqs) - 1, 4).astype(int)]]
    with pbf.Server(solver, 16 << 30, max_scenes=64, cells_per_particle=2.0, max_chunk=64) as srv:
        rids = []
        for k in range(0, len(reqs), 2):
            for r, s in zip(reqs[k:k + 2], scenes[k:k + 2]):
                rids.append(srv.submit(s.params, s.particles, r.steps))
            srv.poll(wait=True)
        srv.run_until_idle()
        assert srv.stats()["completed"] == len(reqs)
        results = {i: srv.result(rids[i]) for i in pick}
    for i in pick:
        r, s = reqs[i], scenes[i]
        with pbf.Batch(solver, 1, s.n, s.params.ncells) as one:
            sid = one.add_scene(s.params, s.particles)
            one.step(r.steps)
            want = one.dump_scene(sid)
        assert inside_walls(s.params, want[0])
        for x, y in zip(results[i], want):
            assert np.array_equal(bits(x), bits(y)), f"request {r.index} ({s.n} particles, {r.steps} steps)"
