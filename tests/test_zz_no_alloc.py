"""pbf_op_sort_pairs_noalloc: the radix sort for callers that cannot allocate
device memory (a host engine whose pool owns every device allocation, or a
per-frame callback where cudaMalloc would stall the device).  Called through
the C-ABI, twice in a row with different inputs, its output must equal that
of pbf_op_sort_pairs (which uses a caller scratch buffer) exactly -- keys and
permutation are integers, so the tolerance is zero.  This file is collected
last so that a failing run stops after every other test has run."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _sort_with_scratch(lib, keys, vals, bits, stream):
    n = keys.shape[0]
    ko = torch.empty(n, dtype=torch.int32, device="cuda")
    vo = torch.empty(n, dtype=torch.int32, device="cuda")
    nbytes = lib.pbf_op_sort_scratch_bytes(n, bits)
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    assert lib.pbf_op_sort_pairs(keys.data_ptr(), vals.data_ptr() if vals is not None else None, n, bits,
                                 ko.data_ptr(), vo.data_ptr(), scratch.data_ptr(), nbytes, stream) == 0
    assert lib.pbf_op_sort_status(scratch.data_ptr(), n, bits, stream) == 0
    return ko, vo


def _sort_noalloc(lib, keys, vals, bits, stream, with_status=True):
    n = keys.shape[0]
    ko = torch.empty(n, dtype=torch.int32, device="cuda")
    vo = torch.empty(n, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.pbf_op_sort_pairs_noalloc(keys.data_ptr(), vals.data_ptr() if vals is not None else None, n,
                                         bits, ko.data_ptr(), vo.data_ptr(),
                                         status.data_ptr() if with_status else None, stream) == 0
    return ko, vo, status


def test_noalloc_sort_matches_scratch_sort_twice(pbf):
    lib = pbf.lib()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2024)
    # (n, key bits, explicit values, status word): 32-bit keys take four
    # digit passes, the largest scratch layout, at the maximum size; one
    # case leaves the status pointer NULL
    cases = [(1 << 20, 18, None, True), (333_333, 13, "vals", True), (1 << 20, 32, "vals", True),
             (1 << 20, 32, None, False)]
    for n, bits, with_vals, with_status in cases:
        keys = torch.from_numpy(rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
                                .view(np.int32)).cuda()
        vals = (torch.from_numpy(rng.integers(0, 1 << 30, n).astype(np.int32)).cuda()
                if with_vals else None)
        want_k, want_v = _sort_with_scratch(lib, keys, vals, bits, stream)
        got_k, got_v, status = _sort_noalloc(lib, keys, vals, bits, stream, with_status)
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        assert torch.equal(got_k, want_k) and torch.equal(got_v, want_v)
        # and it is the stable sort
        order = np.argsort(keys.cpu().numpy().view(np.uint32), kind="stable")
        expect_v = order if vals is None else vals.cpu().numpy()[order]
        assert np.array_equal(got_v.cpu().numpy().view(np.uint32), expect_v.astype(np.uint32))


def test_noalloc_sort_rejects_oversize(pbf):
    lib = pbf.lib()
    n = (1 << 20) + 1
    keys = torch.zeros(n, dtype=torch.int32, device="cuda")
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    rc = lib.pbf_op_sort_pairs_noalloc(keys.data_ptr(), None, n, 8, out.data_ptr(), out.data_ptr(), None,
                                       torch.cuda.current_stream().cuda_stream)
    assert rc == pbf.ERR_INVALID
    assert b"1048576" in lib.pbf_last_error_message()
