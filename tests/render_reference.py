"""NumPy restatement of the headless particle pass (test infrastructure): the sphere-impostor
splat of assets/shaders/draw/particles_3d.slang with the IDL Mac-style colour map of
assets/shaders/draw/colormap.slang, nearest depth wins (LESS_OR_EQUAL, the later particle on ties),
row 0 at NDC y = -1. Pure-Python loops over particles: small cases only."""
from __future__ import annotations

import numpy as np

f32 = np.float32


def mac_style(x):
    x = min(max(f32(x), f32(0)), f32(1))
    h = f32(-7.44992704834645e-01) * x + f32(7.47986634976377e-01)
    i2 = np.fmod(np.fmod(x * f32(256), f32(2)) + f32(2), f32(2))
    v = f32(1) if 0.0 <= i2 < 1.0 else f32(254.0 / 255.0)
    r = g = b = v
    h = h * f32(6)
    i = int(h)
    fr = h - f32(i)
    if i == 1:
        r, b = r * (1 - fr), b * 0
    elif i == 2:
        r, b = r * 0, b * (1 - (1 - fr))
    elif i == 3:
        r, g = r * 0, g * (1 - fr)
    elif i == 4:
        r, g = r * (1 - (1 - fr)), g * 0
    elif i == 5:
        g, b = g * 0, b * (1 - fr)
    else:
        g, b = g * (1 - (1 - fr)), b * 0
    return np.array([r, g, b], np.float64)


def render(pos, vel, mv, pj, width, height, quad_side=0.15, depth_radius=0.15, v_max=6.5):
    MV = np.asarray(mv, np.float64).reshape(4, 4).T  # row-major view of the column-major data
    P = np.asarray(pj, np.float64).reshape(4, 4).T
    hs = 0.5 * quad_side
    light = np.array([0.0, 1.0, 1.0]) / np.sqrt(2.0)
    zbuf = np.full((height, width), np.inf)
    owner = np.full((height, width), -1, np.int64)
    normals = np.zeros((height, width, 3))
    ll, ur = P @ np.array([-hs, -hs, 0, 1]), P @ np.array([hs, hs, 0, 1])
    cx = (2.0 * (np.arange(width) + 0.5)) / width - 1.0
    cy = (2.0 * (np.arange(height) + 0.5)) / height - 1.0
    for i, p in enumerate(pos):
        v = MV @ np.array([p[0], p[1], p[2], 1.0])
        c = P @ v
        wl, wu = c[3] + ll[3], c[3] + ur[3]
        if not (wl > 0 and wu > 0):
            continue
        x0, y0 = (c[0] + ll[0]) / wl, (c[1] + ll[1]) / wl
        x1, y1 = (c[0] + ur[0]) / wu, (c[1] + ur[1]) / wu
        u = (cx[None, :] - x0) / (x1 - x0)
        w = (cy[:, None] - y0) / (y1 - y0)
        nx, ny = np.broadcast_arrays(u * 2 - 1, w * 2 - 1)
        r2 = nx * nx + ny * ny
        inside = r2 <= 1.0
        nz = np.sqrt(np.clip(1.0 - r2, 0.0, None))
        pv = v[:3, None, None] + depth_radius * np.stack([nx, ny, nz])
        cc = np.einsum("ij,jhw->ihw", P, np.concatenate([pv, np.ones((1,) + nx.shape)]))
        d = cc[2] / cc[3]
        ok = inside & (d >= 0) & (d <= 1) & (d <= zbuf)
        zbuf[ok] = d[ok]
        owner[ok] = i
        normals[ok] = np.stack([nx, ny, nz], -1)[ok]
    img = np.zeros((height, width, 4), np.uint8)
    img[..., 3] = 255
    for yx in zip(*np.nonzero(owner >= 0)):
        i = owner[yx]
        col = mac_style(np.linalg.norm(vel[i]) / v_max)
        diff = max(0.0, float(normals[yx] @ light))
        img[yx][:3] = np.round(np.clip(col * diff, 0, 1) * 255).astype(np.uint8)
    return img, owner
