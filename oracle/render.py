"""Test infrastructure: a numpy restatement of the reference's particle
drawing, the oracle for the CUDA renderer (pbf_render).

Follows src/visual/visual.cpp (camera sphere :86-100, look-at :104-125,
perspective and box centring :217-227, clear colour and depth test
:79-83,270-274), src/shaders/particlevertex.glsl (point size 200 / clip.w)
and src/shaders/particlefragment.glsl (sphere normal from gl_PointCoord,
discard outside the disc, colour (|v|, |v|, 1) * clamp(dot(n, (1,1,1)), 0,
1)).  Particles are drawn in input order with a strict depth test, as GL
draws the buffer.

Every value the image depends on is computed in IEEE binary32, one rounded
operation at a time, in the order the CUDA renderer evaluates it (that
translation unit is compiled without contraction, with correctly rounded
division and square root): the camera's trigonometry in double and rounded
to binary32, as the renderer's host code does, then the matrices, the
sprites, the coverage test and the shading.  The CUDA image must equal this
one pixel for pixel.
"""
from __future__ import annotations

import math

import numpy as np

F = np.float32


def _normalize(v):
    l = np.sqrt(F(F(F(v[0] * v[0]) + F(v[1] * v[1])) + F(v[2] * v[2])))
    return [F(v[0] / l), F(v[1] / l), F(v[2] / l)]


def _mat_mul(a, b):
    """Column-major 4x4 product, each entry summed k = 0..3 from zero."""
    out = [F(0)] * 16
    for c in range(4):
        for row in range(4):
            acc = F(0)
            for k in range(4):
                acc = F(acc + F(a[k * 4 + row] * b[c * 4 + k]))
            out[c * 4 + row] = acc
    return out


def view_projection(cam, aspect) -> list:
    """Column-major 16 floats, clip = M * (p, 1) (glm's layout)."""
    phi = math.pi / 180.0 * (float(cam.phi_deg) - 90.0)
    theta = math.pi / 180.0 * (float(cam.theta_deg) + 90.0)
    d = [F(math.sin(theta) * math.cos(phi)), F(math.cos(theta)), F(math.sin(theta) * math.sin(phi))]
    dist = F(cam.distance)
    tgt = [F(t) for t in cam.target[:3]]
    eye = [F(F(d[a] * dist) + tgt[a]) for a in range(3)]
    look = _normalize([F(tgt[a] - eye[a]) for a in range(3)])
    up = [F(0), F(1), F(0)]
    right = _normalize([F(F(look[1] * up[2]) - F(look[2] * up[1])),
                        F(F(look[2] * up[0]) - F(look[0] * up[2])),
                        F(F(look[0] * up[1]) - F(look[1] * up[0]))])
    pup = [F(F(right[1] * look[2]) - F(right[2] * look[1])),
           F(F(right[2] * look[0]) - F(right[0] * look[2])),
           F(F(right[0] * look[1]) - F(right[1] * look[0]))]
    z, o = F(0), F(1)
    view = [right[0], pup[0], F(-look[0]), z, right[1], pup[1], F(-look[1]), z,
            right[2], pup[2], F(-look[2]), z, z, z, z, o]
    trans = [o, z, z, z, z, o, z, z, z, z, o, z, F(-eye[0]), F(-eye[1]), F(-eye[2]), o]
    view = _mat_mul(view, trans)
    f = F(F(1) / F(math.tan(math.pi / 180.0 * float(cam.fovy_deg) / 2.0)))
    zn, zf = F(cam.znear), F(cam.zfar)
    proj = [F(0)] * 16
    proj[0] = F(f / aspect)
    proj[5] = f
    proj[10] = F(F(-(F(zf + zn))) / F(zf - zn))
    proj[11] = F(-1)
    proj[14] = F(F(-(F(F(F(2) * zf) * zn))) / F(zf - zn))
    return _mat_mul(proj, view)


def _sprite(m, half, width, height, maxs, p):
    wx, wy, wz = (F(F(p[a]) + half[a]) for a in range(3))

    def row(r):
        return F(F(F(F(m[r] * wx) + F(m[4 + r] * wy)) + F(m[8 + r] * wz)) + m[12 + r])

    cx, cy, cz, cw = row(0), row(1), row(2), row(3)
    if not (cw > 0) or abs(cx) > cw or abs(cy) > cw or abs(cz) > cw:
        return None
    inv = F(F(1) / cw)
    x = F(F(F(F(cx * inv) + F(1)) * F(0.5)) * width)
    y = F(F(F(F(cy * inv) + F(1)) * F(0.5)) * height)
    zz = F(F(F(cz * inv) + F(1)) * F(0.5))
    s = min(F(F(200) * inv), maxs)
    return x, y, zz, s


def _point_coord(x, y, s, ix, iy):
    h = F(F(0.5) * s)
    u = F(F(F(F(ix) + F(0.5)) - F(x - h)) / s)
    w = F(F(F(y + h) - F(F(iy) + F(0.5))) / s)
    return F(F(u * F(2)) - F(1)), F(F(w * F(2)) - F(1))


def render(pos4: np.ndarray, params, cam, width: int, height: int) -> np.ndarray:
    """pos4: (N, 4) float32 in input order (.w = |v|).  Returns (H, W, 3) uint8, top row first."""
    fw, fh = F(width), F(height)
    m = view_projection(cam, F(fw / fh))
    half = [F(F(-(F(F(params.x_max) - F(params.x_min)))) / F(2)),
            F(F(-(F(F(params.y_max) - F(params.y_min)))) / F(2)),
            F(F(-(F(F(params.z_max) - F(params.z_min)))) / F(2))]
    maxs = F(cam.max_point_size if cam.max_point_size > 0 else 64)
    zbuf = np.full((height, width), np.inf, np.float64)
    owner = np.full((height, width), -1, np.int64)
    sprites = []
    pos = np.asarray(pos4, np.float32)
    for i in range(pos.shape[0]):
        sp = _sprite(m, half, fw, fh, maxs, pos[i, :3])
        sprites.append(sp)
        if sp is None:
            continue
        x, y, z, s = sp
        h = F(F(0.5) * s)
        x0 = max(0, int(np.ceil(F(F(x - h) - F(0.5)))))
        x1 = min(width - 1, int(np.floor(F(F(x + h) - F(0.5)))))
        y0 = max(0, int(np.ceil(F(F(y - h) - F(0.5)))))
        y1 = min(height - 1, int(np.floor(F(F(y + h) - F(0.5)))))
        for iy in range(y0, y1 + 1):
            for ix in range(x0, x1 + 1):
                mx, my = _point_coord(x, y, s, ix, iy)
                if F(F(mx * mx) + F(my * my)) > F(1):
                    continue
                if z < zbuf[iy, ix]:  # strict: the first particle drawn keeps a tie
                    zbuf[iy, ix] = z
                    owner[iy, ix] = i
    img = np.zeros((height, width, 3), np.uint8)
    grey = int(np.rint(F(F(0.05) * F(255))))
    img[:] = grey
    for iy in range(height):
        for ix in range(width):
            i = owner[iy, ix]
            if i < 0:
                continue
            x, y, z, s = sprites[i]
            mx, my = _point_coord(x, y, s, ix, iy)
            l2 = F(F(mx * mx) + F(my * my))
            nz = np.sqrt(max(F(0), F(F(1) - l2)))
            inv = F(F(1) / np.sqrt(max(F(l2 + F(nz * nz)), F(1e-30))))
            cosang = min(max(F(F(F(mx + my) + nz) * inv), F(0)), F(1))
            v = F(pos[i, 3])
            rgb = (F(v * cosang), F(v * cosang), cosang)
            img[iy, ix] = [int(np.rint(F(min(max(c, F(0)), F(1)) * F(255)))) for c in rgb]
    return img[::-1].copy()
