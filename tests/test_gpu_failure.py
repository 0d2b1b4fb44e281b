"""Failure detection without a GPU fault: the radix sort's bounded
look-back wait, run against a predecessor that never publishes, gives up
after its poll limit, reports PBF_ERR_DEVICE through the error flag, and the
CUDA context stays usable (a simulation steps normally afterwards)."""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_context_survives(pbf):
    flag = C.c_uint32()
    t0 = time.perf_counter()
    status = pbf.lib().pbf_selftest_bounded_wait(1 << 16, C.byref(flag))
    elapsed = time.perf_counter() - t0
    assert status == pbf.ERR_DEVICE
    assert flag.value & 1  # the look-back error bit
    assert elapsed < 5.0
    sc = pbf.scenes.dam_break((8, 8, 8), (0.8, 0.8, 0.8), seed=71)
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        sim.step(3)
        pos, _ = sim.dumpData()
    assert np.isfinite(pos).all()
