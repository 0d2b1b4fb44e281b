"""bench.py's host-side helpers (no GPU): the roofline's traffic lines are
present and parseable in the committed profiles for every kernel the bench
can name as dominant, the measured-peak lookup falls back cleanly, the
density-error summary is computed as stated, and the command line lists
its workloads."""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_traffic_lines_for_every_timed_kernel():
    for kernel in bench.ALG_BYTES:
        got = bench.profile_traffic(kernel)
        assert got is not None, kernel
        nbytes, particles = got
        assert nbytes > 0 and particles == 1048576, kernel
    assert bench.profile_traffic("no_such_kernel") is None


def test_algorithmic_bytes_sum_to_the_step_total():
    per_step = {"predict_hash": 1, "sort_onesweep": 1, "cell_offsets": 1, "reorder": 1,
                "lambda": 4, "delta": 4, "vorticity": 1, "xsph_commit": 1}
    cells_64 = 64 ** 3
    assert sum(bench.ALG_BYTES[k] * m for k, m in per_step.items()) == bench.step_bytes(cells_64)
    assert bench.sort_bytes(cells_64) == bench.ALG_BYTES["sort_onesweep"] == 4 + 16 * 2


def test_counting_sort_bytes():
    n, cells = 1 << 20, 64 ** 3
    assert bench.cell_sort_bytes(n, cells) == bench.ALG_BYTES["cell_sort"] == 22
    assert bench.step_bytes(cells, n, counting=True) == 592 - 36 - 8 + 22


def test_sort_passes_follow_the_digit_plan():
    # 9-bit digits only for 9 and 17-18 key bits; 8-bit digits otherwise
    want = {1: 1, 8: 1, 9: 1, 10: 2, 16: 2, 17: 2, 18: 2, 19: 3, 20: 3, 24: 3, 25: 4,
            27: 4, 32: 4}
    assert {b: bench.sort_passes(b) for b in want} == want
    assert bench.sort_key_bits(128 * 128 * 64) == 20 and bench.sort_bytes(128 * 128 * 64) == 52


def test_measured_peaks_has_a_bandwidth():
    p = bench.measured_peaks()
    assert p["hbm_gbs"] > 1000.0 and p["source"] in ("measured", "fallback")


def test_density_error_summary():
    class FakeSim:
        def density(self):
            return np.array([8000.0, 8800.0, 4000.0, 7200.0], np.float32)

    d = bench.density_error_of(FakeSim(), 8000.0, 12)
    assert d["at_step"] == 12
    assert abs(d["max_compression"] - 0.1) < 1e-6
    assert abs(d["mean_compression"] - 0.025) < 1e-6
    # interior: rho >= 0.8 rho0 -> 1.0, 1.1, 0.9
    assert abs(d["mean_abs_interior"] - (0.0 + 0.1 + 0.1) / 3) < 1e-6


def test_command_line_lists_the_workloads():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True,
                         text=True, timeout=60)
    assert out.returncode == 0
    for w in ("single", "large", "batch", "serve", "aux"):
        assert w in out.stdout
