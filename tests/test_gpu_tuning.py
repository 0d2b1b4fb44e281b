"""Launch-shape tuning of the gather passes (pbf_autotune, pbf_set_tuning).

Statement (checked below): every launch shape -- 64/128/256 threads per CTA,
4 or 8 neighbour loads in flight, list build fused with the first lambda or
not, members stored as found or from row masks -- gives BIT-IDENTICAL
steps, and pbf_autotune leaves the simulation's state unchanged, so a tuned
run is bitwise the untuned run.
"""
from __future__ import annotations

import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def shape(pbf, threads, batch, fuse, masked=0):
    t = pbf.Tuning()
    for k in range(6):
        t.threads[k] = threads
        t.batch[k] = batch
    t.fuse_first = fuse
    t.masked_build = masked
    return t


def run(pbf, sc, steps, tuning=None, autotune=0):
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        if tuning is not None:
            sim.set_tuning(tuning)
        if autotune:
            sim.step(2)
            before = sim.dumpData()
            sim.autotune(autotune)
            after = sim.dumpData()
            for x, y in zip(before, after):
                assert np.array_equal(bits(x), bits(y)), "autotune changed the state"
            steps -= 2
        sim.step(steps)
        return sim.dumpData(), (sim.launches_per_step(), sim.tuning().fuse_first)


def test_every_launch_shape_gives_the_same_bits(pbf):
    sc = pbf.scenes.dam_break((16, 14, 12), (0.8, 1.6, 0.8), seed=31)
    small = sc.params.copy()
    small.max_neighbours = 16  # some particles take the re-derived path too
    small.grow_lists = 0
    for prm in (sc.params, small):
        scene = pbf.scenes.Scene(sc.name, prm, sc.particles, 8)
        ref, (launches, default_fuse) = run(pbf, scene, 8)
        for threads, batch, fuse, masked in itertools.product((64, 128, 256), (4, 8), (0, 1),
                                                              (0, 1)):
            got, (n, _) = run(pbf, scene, 8, shape(pbf, threads, batch, fuse, masked))
            for g, r in zip(got, ref):
                assert np.array_equal(bits(g), bits(r)), (threads, batch, fuse, masked)
            assert n == launches + default_fuse - fuse  # fused: one launch fewer


def test_autotune_keeps_state_and_results(pbf):
    sc = pbf.scenes.dam_break((20, 20, 10), (1.6, 1.6, 0.8), seed=32)
    ref, _ = run(pbf, sc, 10)
    got, _ = run(pbf, sc, 10, autotune=2)
    for g, r in zip(got, ref):
        assert np.array_equal(bits(g), bits(r))
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        t = sim.autotune(2).as_dict()
        assert set(t["threads"].values()) <= {64, 128, 256}
        assert set(t["batch"].values()) <= {4, 8}
        assert all(v > 0 for k, v in t["trial_ms"].items())
        assert sim.tuning().as_dict()["threads"] == t["threads"]


def test_invalid_shapes_are_rejected(pbf):
    sc = pbf.scenes.dam_break((6, 6, 6), (0.8, 0.8, 0.8), seed=33)
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        for bad in (shape(pbf, 96, 4, 0), shape(pbf, 128, 6, 0), shape(pbf, 128, 4, 2),
                    shape(pbf, 128, 4, 0, 2)):
            with pytest.raises(pbf.PbfError) as ex:
                sim.set_tuning(bad)
            assert ex.value.status == pbf.ERR_INVALID
        with pytest.raises(pbf.PbfError):
            sim.autotune(0)


def test_batch_autotune_keeps_results(pbf):
    scenes = pbf.scenes.mixed_batch(count=5, n_min=1000, n_max=20000, seed=3)
    cap = (len(scenes), sum(s.n for s in scenes), sum(s.params.ncells for s in scenes))
    out = []
    for tune in (False, True):
        with pbf.Batch(scenes[0].params, *cap) as b:
            ids = [b.add_scene(s.params, s.particles) for s in scenes]
            b.step(3)
            if tune:
                b.autotune(2)
            b.step(5)
            out.append([b.dump_scene(i) for i in ids])
    for a, c in zip(*out):
        for x, y in zip(a, c):
            assert np.array_equal(bits(x), bits(y))


def test_masked_build_with_rows_over_32_candidates(pbf):
    """A block at twice the linear density (spacing h/4: ~64 particles per
    cell, rows of ~190 candidates) makes the masked list build test each row
    in several 32-candidate chunks; fused or not, it gives the lists and
    bits of the build that stores members as it finds them."""
    box, cells = (0.8, 0.8, 0.8), (8, 8, 8)
    p = pbf.scenes.base_params(box, cells)
    p.max_neighbours = 512
    m = 0.25 * pbf.scenes.H
    ps = pbf.generate_block((m, m, m), 16, 16, 16, 0.025, 0.01 * 0.025, pbf.scenes.MASS, 77)
    scene = pbf.scenes.Scene("dense_block", p, ps, 3)
    for fuse in (0, 1):
        out = []
        for masked in (0, 1):
            with pbf.Simulation(scene.params, scene.particles) as sim:
                sim.init()
                sim.set_tuning(shape(pbf, 128, 4, fuse, masked))
                sim.step(1)
                mx, over = sim.neighbour_stats()
                assert mx > 128 and over == 0, (mx, over)
                sim.step(2)
                out.append(sim.dumpData())
        for a, b in zip(*out):
            assert np.array_equal(bits(a), bits(b)), fuse
