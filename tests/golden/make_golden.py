"""Generates the golden vectors in tests/golden/ref_scenarios.npz.

Source of truth: the reference's own live kernels (MrMagne/position-based-
fluids src/kernels/*.cl) compiled as C++ by oracle/build.py and run by
oracle/ref_launch.cpp, in the step order of src/Simulation.cpp:455-576,
with update_cells.cl launched in ascending work-item order.  Inputs are the
reference's scenario files (assets/scenarios/*.par + *.in), read here and
stored in the fixture so that the tests need neither the reference tree nor
its build.

For every scenario and every listed step count K the fixture stores, after K
steps from the scenario's initial state: positions and velocities (dumpData
layout), predicted positions (.w = density of the last lambda pass), lambda
of the last iteration, and the cell of every particle as recorded in the
reference's linked cell lists of the last step.

Usage (the reference checkout in PBF_REFERENCE_ROOT, see oracle/build.py):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

from oracle.build import REFERENCE_SCENARIOS as SCENARIOS  # noqa: E402  (PBF_REFERENCE_ROOT)
OUT = Path(__file__).resolve().parent / "ref_scenarios.npz"

# name -> step counts.  box.in goes non-finite in the reference's own
# kernels at step 3 (27 particles 0.001 apart with h = 0.01), after which
# its cell hash indexes out of bounds, so it stops at 2 steps.
PLAN = {
    "two": [1, 5, 20],
    "two_updown": [1, 5, 20],
    "box_small": [1, 5, 20],
    "27": [1, 5, 20],
    "box": [1, 2],
    "box_big": [1, 5],
    "dam": [1, 5],
    "dam_miles": [1, 3],
}

CONFIG_FIELDS = ["x_min", "x_max", "y_min", "y_max", "z_min", "z_max", "x_n", "y_n", "z_n",
                 "timestep_length", "rest_density"]


def cell_of_particle(cells: np.ndarray, lst: np.ndarray, n: int) -> np.ndarray:
    out = np.full(n, -1, np.int64)
    for c, members in oracle.cells_from_lists(cells, lst).items():
        out[members] = c
    if (out < 0).any():
        raise RuntimeError("particle missing from the reference cell lists")
    return out.astype(np.uint32)


def main() -> None:
    if not oracle.reference_available():
        raise SystemExit("the reference's kernels could not be built here")
    data = {}
    for name, steps in PLAN.items():
        cfg = oracle.read_par(SCENARIOS / f"{name}.par")
        pos, vel = oracle.read_in(SCENARIOS / f"{name}.in")
        data[f"{name}/config"] = np.array([getattr(cfg, f) for f in CONFIG_FIELDS], np.float32)
        data[f"{name}/pos0"] = pos
        data[f"{name}/vel0"] = vel
        data[f"{name}/steps"] = np.array(steps, np.int32)
        for k in steps:
            p, v, pred, sc, cells, lst = oracle.reference_steps(cfg, pos, vel, k, threads=8)
            if not (np.isfinite(p).all() and np.isfinite(v).all()):
                raise RuntimeError(f"{name} after {k} steps is not finite")
            data[f"{name}/k{k}/pos"] = p
            data[f"{name}/k{k}/vel"] = v
            data[f"{name}/k{k}/pred"] = pred
            data[f"{name}/k{k}/scaling"] = sc
            data[f"{name}/k{k}/cell"] = cell_of_particle(cells, lst, p.shape[0])
        print(name, pos.shape[0], steps)
    np.savez_compressed(OUT, **data)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
