"""Density error over a 500-step dam break (32,768 particles, 32^3 block in a
1.6 x 1.6 x 3.2 box, paper equations), sampled every 10 steps from the
density of each step's last lambda pass.

Stated bounds, over all samples:
  * mean compression  mean(max(rho/rho0 - 1, 0))        <= 0.10
  * max compression   max(rho/rho0 - 1)                  <= 1.00
  * mean |rho/rho0 - 1| over particles away from the free surface
    (rho >= 0.8 rho0)                                    <= 0.12
and over the settled last 100 steps mean compression <= 0.06; every position
stays finite and inside the walls.  The FP64 oracle on the same scene peaks
at 0.087 / 0.48 / 0.091 during the splash (steps 30-40) and settles at about
0.04 mean compression (4 iterations with relaxation 600 are soft).
"""
from __future__ import annotations

import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_density_error_bounds_over_500_steps(pbf):
    sc = pbf.scenes.config_small()
    rho0 = sc.params.rest_density
    m = sc.params.wall_margin
    box = np.array([sc.params.x_max, sc.params.y_max, sc.params.z_max])
    stats = []
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        for k in range(50):
            sim.step(10)
            rho = sim.density() / rho0
            comp = np.maximum(rho - 1.0, 0.0)
            interior = rho >= 0.8
            stats.append({
                "step": 10 * (k + 1),
                "mean_compression": float(comp.mean()),
                "max_compression": float(comp.max()),
                "mean_abs_interior": float(np.abs(rho[interior] - 1.0).mean()) if interior.any() else 0.0,
            })
        pos, vel = sim.dumpData()
    print(json.dumps({"density_error_500_steps": stats[-1], "worst": {
        "mean_compression": max(s["mean_compression"] for s in stats),
        "max_compression": max(s["max_compression"] for s in stats),
        "mean_abs_interior": max(s["mean_abs_interior"] for s in stats)}}))
    assert np.isfinite(pos).all() and np.isfinite(vel).all()
    tol = 1e-4
    assert (pos[:, :3] >= m - tol).all() and (pos[:, :3] <= box - m + tol).all()
    assert max(s["mean_compression"] for s in stats) <= 0.10
    assert max(s["max_compression"] for s in stats) <= 1.00
    assert max(s["mean_abs_interior"] for s in stats) <= 0.12
    assert max(s["mean_compression"] for s in stats if s["step"] > 400) <= 0.06
