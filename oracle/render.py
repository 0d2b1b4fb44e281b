"""Test infrastructure: a numpy restatement of the reference's particle
drawing, the oracle for the CUDA renderer (pbf_render).

Follows src/visual/visual.cpp (camera sphere :86-100, look-at :104-125,
perspective and box centring :217-227, clear colour and depth test
:79-83,270-274), src/shaders/particlevertex.glsl (point size 200 / clip.w)
and src/shaders/particlefragment.glsl (sphere normal from gl_PointCoord,
discard outside the disc, colour (|v|, |v|, 1) * clamp(dot(n, (1,1,1)), 0,
1)).  Particles are drawn in input order with a strict depth test, as GL
draws the buffer.  Arithmetic in float32 where the GPU path uses float.
"""
from __future__ import annotations

import math

import numpy as np

F = np.float32


def view_projection(cam, aspect: float) -> np.ndarray:
    """Column-major-equivalent 4x4 (as a numpy row-major matrix M, clip = M @ p)."""
    phi = math.pi / 180.0 * (cam.phi_deg - 90.0)
    theta = math.pi / 180.0 * (cam.theta_deg + 90.0)
    d = np.array([math.sin(theta) * math.cos(phi), math.cos(theta), math.sin(theta) * math.sin(phi)], F)
    eye = d * F(cam.distance) + np.array(cam.target[:], F)
    look = np.array(cam.target[:], F) - eye
    look = look / np.sqrt(np.sum(look * look, dtype=F))
    up = np.array([0, 1, 0], F)
    right = np.cross(look, up).astype(F)
    right = right / np.sqrt(np.sum(right * right, dtype=F))
    pup = np.cross(right, look).astype(F)
    view = np.eye(4, dtype=F)
    view[0, :3], view[1, :3], view[2, :3] = right, pup, -look
    trans = np.eye(4, dtype=F)
    trans[:3, 3] = -eye
    f = F(1.0 / math.tan(math.pi / 180.0 * cam.fovy_deg / 2.0))
    zn, zf = F(cam.znear), F(cam.zfar)
    proj = np.zeros((4, 4), F)
    proj[0, 0] = f / F(aspect)
    proj[1, 1] = f
    proj[2, 2] = -(zf + zn) / (zf - zn)
    proj[3, 2] = -1
    proj[2, 3] = -(F(2) * zf * zn) / (zf - zn)
    return (proj @ (view @ trans)).astype(F)


def render(pos4: np.ndarray, params, cam, width: int, height: int) -> np.ndarray:
    """pos4: (N, 4) float32 in input order (.w = |v|).  Returns (H, W, 3) uint8, top row first."""
    M = view_projection(cam, width / height)
    half = np.array([-(params.x_max - params.x_min) / 2, -(params.y_max - params.y_min) / 2,
                     -(params.z_max - params.z_min) / 2], F)
    zbuf = np.full((height, width), np.inf, np.float64)
    owner = np.full((height, width), -1, np.int64)
    sprites = []
    maxs = F(cam.max_point_size if cam.max_point_size > 0 else 64)
    for i in range(pos4.shape[0]):
        w = np.append(pos4[i, :3].astype(F) + half, F(1))
        c = (M @ w).astype(F)
        if not (c[3] > 0) or abs(c[0]) > c[3] or abs(c[1]) > c[3] or abs(c[2]) > c[3]:
            sprites.append(None)
            continue
        inv = F(1) / c[3]
        x = (c[0] * inv + F(1)) * F(0.5) * F(width)
        y = (c[1] * inv + F(1)) * F(0.5) * F(height)
        z = (c[2] * inv + F(1)) * F(0.5)
        s = min(F(200) * inv, maxs)
        sprites.append((x, y, z, s))
        x0 = max(0, math.ceil(x - s / 2 - 0.5)); x1 = min(width - 1, math.floor(x + s / 2 - 0.5))
        y0 = max(0, math.ceil(y - s / 2 - 0.5)); y1 = min(height - 1, math.floor(y + s / 2 - 0.5))
        for iy in range(y0, y1 + 1):
            for ix in range(x0, x1 + 1):
                mx = ((ix + F(0.5)) - (x - F(0.5) * s)) / s * 2 - 1
                my = ((y + F(0.5) * s) - (iy + F(0.5))) / s * 2 - 1
                if mx * mx + my * my > 1:
                    continue
                if z < zbuf[iy, ix]:
                    zbuf[iy, ix] = z
                    owner[iy, ix] = i
    img = np.full((height, width, 3), 0.05, np.float64)
    for iy in range(height):
        for ix in range(width):
            i = owner[iy, ix]
            if i < 0:
                continue
            x, y, z, s = sprites[i]
            mx = ((ix + F(0.5)) - (x - F(0.5) * s)) / s * 2 - 1
            my = ((y + F(0.5) * s) - (iy + F(0.5))) / s * 2 - 1
            nz = math.sqrt(max(0.0, 1.0 - (mx * mx + my * my)))
            cosang = min(max((mx + my + nz) / math.sqrt(mx * mx + my * my + nz * nz), 0.0), 1.0)
            v = float(pos4[i, 3])
            img[iy, ix] = (v * cosang, v * cosang, cosang)
    out = np.rint(np.clip(img, 0, 1) * 255).astype(np.uint8)
    return out[::-1].copy()
