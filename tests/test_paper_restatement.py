"""The FP64 paper-equation oracle against a second restatement of the same
equations, written here from Macklin & Mueller, "Position Based Fluids"
(ACM TOG 32(4), 2013), Algorithm 1, with the choices the oracle documents
(number densities, the self term W(0), s_corr = -k h^2 (W(r)/W(dq h))^n,
walls `wall_margin` inside the box, 1/rho_j weights in the velocity terms,
neighbour sets from the predicted positions at the step start).

This restatement shares no code with the oracle: it is dense numpy over all
particle pairs (no cells, no lists), summing every term with numpy's
reductions instead of the oracle's per-particle loops, so the two agree only
up to the rounding of different summation orders.  A misreading common to
both cannot show here; an error in either implementation can.
"""
from __future__ import annotations

import math

import numpy as np
import pytest


def paper_step(prm, x, v, wave=0.0):
    """One step of Algorithm 1 in float64 on (n, 3) positions and velocities."""
    h = prm.h
    h2 = h * h
    poly6 = 315.0 / (64.0 * math.pi * h ** 9)
    spiky = 45.0 / (math.pi * h ** 6)
    rho0, dt = prm.rest_density, prm.dt
    dq2 = (prm.scorr_dq * h) ** 2
    lo = np.array(prm.box_min[:], float) + prm.wall_margin
    lo[0] += wave
    hi = np.array(prm.box_max[:], float) - prm.wall_margin

    v = v.copy()
    v[:, 1] += dt * prm.gravity_y                      # line 2: v* = v + dt f_ext
    d = dt * v
    p = x + d                                          # line 3: x* = x + dt v*
    sep = p[:, None, :] - p[None, :, :]
    r2 = (sep ** 2).sum(-1)
    listed = (r2 > 0) & (r2 < h2)                      # line 6: N_i(x*)

    def pairs(p):
        sep = p[:, None, :] - p[None, :, :]
        r2 = (sep ** 2).sum(-1)
        on = listed & (r2 > 0) & (r2 < h2)             # W = 0 beyond h
        r = np.sqrt(np.where(on, r2, 1.0))
        g = np.where(on, -spiky * (h - r) ** 2 / r, 0.0)[..., None] * sep   # grad_i W(p_i - p_j)
        w = np.where(on, poly6 * (h2 - r2) ** 3, 0.0)
        return sep, r2, on, g, w

    for _ in range(prm.iterations):                    # lines 8-19
        sep, r2, on, g, w = pairs(p)
        rho = poly6 * h2 ** 3 + w.sum(1)               # eq. 2, self term included
        c = rho / rho0 - 1.0                           # eq. 1
        grad_self = g.sum(1)                           # eq. 8, k = i
        den = ((grad_self ** 2).sum(-1) + (g ** 2).sum((1, 2))) / rho0 ** 2
        lam = -c / (den + prm.relax_eps)               # eq. 11
        scorr = np.where(on, -prm.scorr_k * h2 * ((h2 - r2) / (h2 - dq2)) ** (3 * prm.scorr_n), 0.0)
        dp = ((lam[:, None] + lam[None, :] + scorr)[..., None] * g).sum(1) / rho0   # eq. 14
        q = np.clip(x + d + dp, lo, hi)                # collision response
        d = q - x
        p = x + d                                      # line 17: x* = x* + dp
    vel = d / dt                                       # line 21
    sep, r2, on, g, w = pairs(p)
    inv = 1.0 / rho                                    # densities of the last lambda pass
    u = vel[None, :, :] - vel[:, None, :]              # v_j - v_i
    omega = (inv[None, :, None] * np.cross(g, u)).sum(1)           # eq. 15
    om = np.sqrt((omega ** 2).sum(-1))
    eta = ((inv[None, :] * (om[None, :] - om[:, None]))[..., None] * g).sum(1)
    el = np.sqrt((eta ** 2).sum(-1))
    n_hat = np.where(el[:, None] > 0, eta / np.where(el > 0, el, 1.0)[:, None], 0.0)
    force = prm.vort_eps * np.cross(n_hat, omega)      # eq. 16
    xsph = ((w * inv[None, :])[..., None] * u).sum(1)  # eq. 17
    return p, vel + dt * force + prm.xsph_c * xsph


def steps(prm, x, v, n, wave=0.0):
    for _ in range(n):
        x, v = paper_step(prm, x, v, wave)
    return x, v


@pytest.mark.parametrize("case", ["rest", "moving", "wave"])
def test_oracle_matches_dense_restatement(oracle_mod, case):
    cfg, pos, vel = oracle_mod.dam_break_scene((8, 8, 8), (0.8, 0.8, 0.8))
    prm = oracle_mod.benchmark_paper_params(cfg)
    pos = np.asarray(pos, np.float64).reshape(-1, 4)
    vel = np.asarray(vel, np.float64).reshape(-1, 4)
    wave = 0.0
    if case != "rest":
        # a state in motion, with vorticity and XSPH terms at work
        pos, vel, *_ = oracle_mod.paper_steps_f64(prm, pos, vel, 6, threads=1)
    if case == "wave":
        wave = 0.004  # the x-min wall moved 0.04 h into the block
    got, gvel, *_ = oracle_mod.paper_steps_f64(prm, pos, vel, 3, wave=wave, threads=1)
    want, wvel = steps(prm, pos[:, :3], vel[:, :3], 3, wave)
    h = prm.h
    assert np.abs(got[:, :3] - want).max() < 1e-11 * h
    vmax = max(1.0, np.abs(wvel).max())
    assert np.abs(gvel[:, :3] - wvel).max() < 1e-10 * vmax
    if case == "moving":
        assert np.abs(wvel).max() > 0.1  # the comparison saw motion
