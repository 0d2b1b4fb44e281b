"""The counting sort of cell keys (the PAPER step's sort, pbf_op_sort_cells):
the stable permutation and the CSR cell offsets, bit-exact against numpy's
stable argsort and against the onesweep radix sort, for every path a cell
can take -- up to 16 keys (sorted by one thread), 17..64 (one warp),
65..8192 (shared memory), more (a bitmap of the indices) -- and the whole
step with either sort giving the same bits."""
from __future__ import annotations

import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def sort_cells(pbf, keys: np.ndarray, ncells: int):
    n = keys.shape[0]
    dk = dev(keys.astype(np.uint32).view(np.int32)) if n else torch.empty(1, dtype=torch.int32,
                                                                          device="cuda")
    off = torch.full((ncells + 1,), -1, dtype=torch.int32, device="cuda")
    sk = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    pm = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    nbytes = pbf.op_sort_cells_scratch_bytes(n, ncells)
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    pbf.op_sort_cells(dk.data_ptr(), n, ncells, off.data_ptr(), sk.data_ptr(), pm.data_ptr(),
                      scratch.data_ptr(), nbytes, st)
    pbf.op_sort_cells_status(scratch.data_ptr(), n, ncells, st)
    torch.cuda.synchronize()
    return (off.cpu().numpy().view(np.uint32), sk.cpu().numpy().view(np.uint32)[:n],
            pm.cpu().numpy().view(np.uint32)[:n])


def expect(keys, ncells):
    perm = np.argsort(keys, kind="stable").astype(np.uint32)
    off = np.zeros(ncells + 1, np.uint32)
    off[1:] = np.cumsum(np.bincount(keys, minlength=ncells))
    return off, keys[perm], perm


def make(kind, n, ncells, rng):
    if kind == "uniform":
        return rng.integers(0, ncells, n).astype(np.uint32)
    if kind == "cells8":  # a sorted lattice, one step later: runs of 8, 2% moved
        k = np.repeat(np.arange(ncells, dtype=np.uint32), 8)[:n]
        moved = rng.integers(0, n, n // 50)
        k[moved] = np.minimum(k[moved] + rng.integers(0, 3, moved.size), ncells - 1)
        return k
    if kind == "descending":  # every cell's keys arrive in reverse order
        return np.sort(rng.integers(0, ncells, n).astype(np.uint32))[::-1].copy()
    if kind == "one_cell":
        return np.full(n, ncells // 2, np.uint32)
    if kind == "big_cells":  # 17..8192 keys per cell
        return rng.integers(0, ncells, n).astype(np.uint32)
    if kind == "mixed":  # a few huge cells, some big, many small, shuffled
        huge = np.full(20_000, 3, np.uint32)
        big = np.repeat(np.arange(10, 40, dtype=np.uint32), 500)
        small = rng.integers(100, ncells, n - huge.size - big.size).astype(np.uint32)
        k = np.concatenate([huge, big, small])
        return k[rng.permutation(k.size)]
    raise ValueError(kind)


CASES = [
    ("uniform_1m", "uniform", 1 << 20, 64 ** 3),
    ("lattice_1m", "cells8", 1 << 20, 64 ** 3),
    ("descending", "descending", 300_001, 5000),
    ("one_cell_huge", "one_cell", 100_000, 7),
    ("big_cells", "big_cells", 200_000, 50),
    ("warp_cells", "uniform", 300_000, 10_000),      # ~30 per cell: one warp each
    ("around_64", "uniform", 640_000, 10_000),       # either side of 64 per cell
    ("mixed", "mixed", 400_000, 100_000),
    ("one_key", "uniform", 1, 3),
    ("one_cell_grid", "uniform", 5000, 1),
    ("ragged_tiles", "uniform", 4097, 2049),
    ("ragged_scan_tiles", "uniform", 60_000, 3 * 8192 + 2049 + 5),
    ("many_scan_tiles", "uniform", 1 << 20, 3_000_001),
]


@pytest.mark.parametrize("name,kind,n,ncells", CASES, ids=[c[0] for c in CASES])
def test_sort_cells_is_the_stable_permutation(pbf, name, kind, n, ncells):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    keys = make(kind, n, ncells, rng)
    off, sk, perm = sort_cells(pbf, keys, ncells)
    want_off, want_sk, want_perm = expect(keys, ncells)
    assert np.array_equal(off, want_off)
    assert np.array_equal(perm, want_perm)
    assert np.array_equal(sk, want_sk)


def test_sort_cells_empty(pbf):
    off, sk, perm = sort_cells(pbf, np.zeros(0, np.uint32), 9)
    assert np.array_equal(off, np.zeros(10, np.uint32))


def test_sort_cells_reports_a_key_outside_the_grid(pbf):
    keys = np.array([0, 5, 2, 9, 1], np.uint32)  # 9 is not below ncells = 6
    with pytest.raises(pbf.PbfError):
        sort_cells(pbf, keys, 6)


def test_sort_cells_equals_the_radix_sort(pbf):
    rng = np.random.default_rng(5)
    n, ncells = 500_000, 64 ** 3
    keys = make("cells8", n, ncells, rng)
    off, sk, perm = sort_cells(pbf, keys, ncells)
    dk = dev(keys.view(np.int32))
    ko = torch.empty(n, dtype=torch.int32, device="cuda")
    vo = torch.empty(n, dtype=torch.int32, device="cuda")
    nbytes = pbf.op_sort_scratch_bytes(n, 18)
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    pbf.op_sort_pairs(dk.data_ptr(), None, n, 18, ko.data_ptr(), vo.data_ptr(), scratch.data_ptr(),
                      nbytes, st)
    pbf.op_sort_status(scratch.data_ptr(), n, 18, st)
    torch.cuda.synchronize()
    assert np.array_equal(vo.cpu().numpy().view(np.uint32), perm)
    assert np.array_equal(ko.cpu().numpy().view(np.uint32), sk)


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _run(pbf, params, particles, steps, radix):
    with pbf.Simulation(params, particles) as sim:
        sim.init()
        t = sim.tuning()
        t.radix_sort = 1 if radix else 0
        sim.set_tuning(t)
        sim.step(steps)
        pos, vel = sim.dumpData()
        cells = sim.cells()
        dens = sim.density()
    return pos, vel, dens, cells


def _dense_cell(pbf):
    """9,261 particles (21^3 at 4 mm) inside one cell of h = 0.1 m: a cell
    the counting sort orders through its bitmap path."""
    box = (0.8, 0.8, 0.8)
    cells = tuple(int(round(b / pbf.scenes.H)) for b in box)
    p = pbf.scenes.base_params(box, cells)
    p.grow_lists = 0
    ps = pbf.generate_block((0.31, 0.31, 0.31), 21, 21, 21, 0.004, 0.0, pbf.scenes.MASS, 7)
    return p, ps


@pytest.mark.parametrize("case", ["dam_break", "dense_block", "one_dense_cell"])
def test_step_with_counting_sort_equals_radix_sort(pbf, case):
    if case == "dam_break":
        sc = pbf.scenes.dam_break((24, 20, 16), (1.6, 1.6, 1.6), seed=61)
        params, particles, steps = sc.params, sc.particles, 6
    elif case == "dense_block":  # 64 particles per cell: the shared-memory path
        box = (1.6, 1.6, 1.6)
        cells = tuple(int(round(b / pbf.scenes.H)) for b in box)
        params = pbf.scenes.base_params(box, cells)
        params.rest_density = 1.0 / 0.025 ** 3
        params.max_neighbours = 512
        particles = pbf.generate_block((0.5, 0.5, 0.5), 16, 16, 16, 0.025, 0.0002,
                                       pbf.scenes.MASS / 64, 62)
        steps = 2
    else:
        params, particles = _dense_cell(pbf)
        steps = 1
    a = _run(pbf, params, particles, steps, radix=False)
    b = _run(pbf, params, particles, steps, radix=True)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(_bits(x), _bits(y)), case
    for x, y in zip(a[3], b[3]):
        assert np.array_equal(x, y), case


def test_batch_with_counting_sort_equals_radix_sort(pbf):
    scenes = pbf.scenes.mixed_batch(count=6, n_min=1000, n_max=30000, seed=63)
    cap = (len(scenes), sum(s.n for s in scenes), sum(s.params.ncells for s in scenes))
    out = []
    for radix in (False, True):
        with pbf.Batch(scenes[0].params, *cap) as b:
            ids = [b.add_scene(s.params, s.particles) for s in scenes]
            t = b.tuning()
            t.radix_sort = 1 if radix else 0
            b.set_tuning(t)
            b.step(4)
            b.remove_scene(ids[2])  # a new layout: fewer cells, the same scratch
            b.step(3)
            out.append([b.dump_scene(i) for i in ids if i != ids[2]])
    for x, y in zip(*out):
        for a, c in zip(x, y):
            assert np.array_equal(_bits(a), _bits(c))
