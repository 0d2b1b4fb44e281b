"""Neighbour-structure operators on the GPU, through the C-ABI, bit-exact
against the oracle: cell hash (update_cells.cl:10-15), the stable radix sort
of (cell, particle index) keys (the intent of calc_hash.cl + radix_*.cl) and
the inclusive cell ranges (init_cells.cl + find_cells.cl)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_sort(pbf, keys: np.ndarray, key_bits: int, vals: np.ndarray | None = None):
    n = keys.shape[0]
    dk = dev(keys.astype(np.int32).view(np.int32))
    dv = dev(vals.astype(np.int32)) if vals is not None else None
    ko = torch.empty(n, dtype=torch.int32, device="cuda")
    vo = torch.empty(n, dtype=torch.int32, device="cuda")
    nbytes = pbf.op_sort_scratch_bytes(n, key_bits)
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    pbf.op_sort_pairs(dk.data_ptr(), dv.data_ptr() if dv is not None else None, n, key_bits,
                      ko.data_ptr(), vo.data_ptr(), scratch.data_ptr(), nbytes, stream)
    pbf.op_sort_status(scratch.data_ptr(), n, key_bits, stream)
    torch.cuda.synchronize()
    return ko.cpu().numpy().view(np.uint32), vo.cpu().numpy().view(np.uint32)


CASES = [
    ("uniform18", 1 << 20, 18, "uniform"),
    ("tile_minus", 4095, 13, "uniform"),
    ("tile", 4096, 13, "uniform"),
    ("tile_plus", 4097, 13, "uniform"),
    ("one", 1, 5, "uniform"),
    ("all_equal", 100_000, 18, "equal"),
    ("sorted", 300_001, 20, "sorted"),
    ("reverse", 300_001, 20, "reverse"),
    ("bits1", 50_000, 1, "uniform"),
    ("bits8", 50_000, 8, "uniform"),
    ("bits9", 50_000, 9, "uniform"),
    ("bits24", 200_000, 24, "uniform"),
    ("bits32", 200_000, 32, "uniform"),
    ("clustered", 1 << 20, 18, "clustered"),
    # the plans around the 9-bit ones (9 and 17-18 bits): two 8-bit passes
    # (10), two 9-bit (17), three 8-bit (19, 20), four 8-bit (27-31)
    ("bits10", 50_000, 10, "uniform"),
    ("bits17", 200_000, 17, "uniform"),
    ("bits19", 200_000, 19, "uniform"),
    ("bits20_tile_plus", 4097, 20, "uniform"),
    ("bits27", 200_000, 27, "uniform"),
    ("bits30", 200_000, 30, "uniform"),
    ("bits31", 200_000, 31, "uniform"),
    ("clustered20", 1 << 20, 20, "clustered"),
]


def make_keys(kind, n, bits, rng):
    hi = (1 << bits) if bits < 32 else (1 << 32)
    if kind == "uniform":
        k = rng.integers(0, hi, n, dtype=np.uint64)
    elif kind == "equal":
        k = np.full(n, hi // 3, np.uint64)
    elif kind == "sorted":
        k = np.sort(rng.integers(0, hi, n, dtype=np.uint64))
    elif kind == "reverse":
        k = np.sort(rng.integers(0, hi, n, dtype=np.uint64))[::-1]
    else:  # runs of equal keys, as cells of a sorted particle set look
        k = np.repeat(rng.integers(0, hi, n // 8 + 1, dtype=np.uint64), 8)[:n]
        k = np.sort(k)
        k[rng.integers(0, n, n // 50)] = rng.integers(0, hi, n // 50, dtype=np.uint64)
    return k.astype(np.uint32)


@pytest.mark.parametrize("name,n,bits,kind", CASES, ids=[c[0] for c in CASES])
def test_sort_pairs_is_the_stable_permutation(pbf, name, n, bits, kind):
    rng = np.random.default_rng(hash(name) & 0xFFFF)
    keys = make_keys(kind, n, bits, rng)
    sk, perm = gpu_sort(pbf, keys, bits)
    want = np.argsort(keys, kind="stable").astype(np.uint32)
    assert np.array_equal(perm, want)
    assert np.array_equal(sk, keys[want])


def test_digit_widths_give_the_same_permutation(pbf):
    """18-bit keys sorted as 18 bits (two 9-bit passes), 20 and 24 bits
    (three 8-bit passes), 30 and 32 bits (four 8-bit passes): one stable
    permutation."""
    rng = np.random.default_rng(7)
    keys = make_keys("clustered", 500_000, 18, rng)
    first = gpu_sort(pbf, keys, 18)
    for bits in (20, 24, 30, 32):
        got = gpu_sort(pbf, keys, bits)
        assert np.array_equal(got[0], first[0]) and np.array_equal(got[1], first[1]), bits


def test_sort_pairs_carries_values(pbf):
    rng = np.random.default_rng(1)
    n = 123_457
    keys = rng.integers(0, 1 << 16, n).astype(np.uint32)
    vals = rng.integers(0, 1 << 31, n).astype(np.uint32)
    sk, sv = gpu_sort(pbf, keys, 16, vals)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(sk, keys[order]) and np.array_equal(sv, vals[order])


def test_sort_matches_oracle_on_cell_hashes(pbf, oracle_mod):
    sc = pbf.scenes.config_small()
    p = sc.params
    pred = np.zeros((sc.n, 4), np.float32)
    pred[:, :3] = sc.particles["x"]
    cfg = oracle_mod.Config(p.x_min, p.x_max, p.y_min, p.y_max, p.z_min, p.z_max, p.x_n, p.y_n, p.z_n,
                            p.time_step_length, p.rest_density)
    # paper-mode grid: raw cell lengths (no 6-digit rounding); here they agree
    h_or = oracle_mod.cell_hash(cfg, pred)
    dpred = dev(pred)
    dh = torch.empty(sc.n, dtype=torch.int32, device="cuda")
    pbf.op_cell_hash(p, dpred.data_ptr(), sc.n, dh.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    h_gpu = dh.cpu().numpy().view(np.uint32)
    assert np.array_equal(h_gpu, h_or)
    sk_o, perm_o = oracle_mod.sort_cells(h_or)
    sk, perm = gpu_sort(pbf, h_gpu, 13)
    assert np.array_equal(perm, perm_o) and np.array_equal(sk, sk_o)
    # offsets and inclusive ranges
    nc = p.ncells
    off = torch.empty(nc + 1, dtype=torch.int32, device="cuda")
    fl = torch.empty(2 * nc, dtype=torch.int32, device="cuda")
    dsk = dev(sk.view(np.int32))
    st = torch.cuda.current_stream().cuda_stream
    pbf.op_cell_offsets(dsk.data_ptr(), sc.n, nc, off.data_ptr(), st)
    pbf.op_find_cells(off.data_ptr(), nc, fl.data_ptr(), st)
    torch.cuda.synchronize()
    offs = off.cpu().numpy()
    assert offs[0] == 0 and offs[-1] == sc.n and (np.diff(offs) >= 0).all()
    assert np.array_equal(np.diff(offs), np.bincount(sk, minlength=nc))
    assert np.array_equal(fl.cpu().numpy().reshape(nc, 2), oracle_mod.find_cells(sk_o, nc))


def test_hash_ref_compat_grid_matches_reference_lists(pbf, golden, oracle_mod):
    """The reference-constant grid (6-digit constants) reproduces the cell of
    every particle recorded in the reference's own linked lists."""
    from conftest import oracle_config, pbf_params_from_config

    for name in ["dam", "dam_miles", "box_big", "27"]:
        cfgv = golden[f"{name}/config"]
        p = pbf_params_from_config(pbf, cfgv, pbf.MODE_REF_COMPAT)
        cfg = oracle_config(oracle_mod, cfgv)
        dt = oracle_mod.ref_constants(cfg)[12]
        pos0, vel0 = golden[f"{name}/pos0"], golden[f"{name}/vel0"]
        v = vel0.copy()
        v[:, 1] = v[:, 1] + dt * np.float32(-9.81)
        pred = pos0.copy()
        pred[:, :3] = pos0[:, :3] + dt * v[:, :3]
        dh = torch.empty(pred.shape[0], dtype=torch.int32, device="cuda")
        dpred = dev(pred)
        pbf.op_cell_hash(p, dpred.data_ptr(), pred.shape[0], dh.data_ptr(),
                         torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert np.array_equal(dh.cpu().numpy().view(np.uint32), golden[f"{name}/k1/cell"]), name


@pytest.mark.parametrize("mode", ["paper", "ref_compat"])
def test_step_cell_ranges_on_a_sparse_grid(pbf, oracle_mod, mode):
    """The step's cell offsets (every key boundary writes the run of cells it
    starts; runs over 64 cells are queued in chunks of at most 4096 and filled
    by a second kernel) against the inclusive ranges of the sorted keys: a
    small block in the corner of a 16 x 16 x 64-cell box leaves empty runs of
    thousands of cells."""
    m = pbf.MODE_PAPER if mode == "paper" else pbf.MODE_REF_COMPAT
    p = pbf.scenes.base_params((1.6, 1.6, 6.4), (16, 16, 64), mode=m)
    ps = pbf.scenes.block((0.1, 0.1, 0.1), (10, 6, 12), seed=44)
    with pbf.Simulation(p, ps) as sim:
        sim.init()
        sim.step(2)
        hsh, _, rng = sim.cells()
    nc = p.ncells
    sk = np.sort(hsh)
    assert np.array_equal(rng, oracle_mod.find_cells(sk, nc))
    empty = rng[:, 0] < 0
    runs = np.diff(np.flatnonzero(np.diff(np.r_[0, empty.astype(np.int8), 0]) != 0))[::2]
    assert runs.max() > 4096  # the queued, chunked path ran
