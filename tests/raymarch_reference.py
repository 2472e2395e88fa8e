"""NumPy restatement of the density raymarch and of the density grid (test infrastructure).

raymarch(): assets/shaders/draw/raymarch.slang as DensityRaymarchDrawPipeline::Draw
(src/pipelines/raymarch_pipeline.cpp:62-115) draws it: the field's box rasterised with culling off
and a LESS_OR_EQUAL depth test (each pixel starts on the face it sees first), fixed steps while
inside the box (ComputeForwardLightRaymarch, raymarch.slang:60-80), emission
colormap(d * 5) * d * 200 (DensityAtPosition, :50-58; colormap.slang IDL Mac style), the sum
clamped to [0, 1] (a UNORM draw image) and blended with SRC_ALPHA / ONE_MINUS_SRC_ALPHA for
colour and ONE / ONE_MINUS_SRC_ALPHA for alpha (src/gfx/vk_util.cpp:343-356). The field is
sampled trilinearly at uvw = 0.5 (p / half + 1) with texel centres at (i + 0.5) / n and REPEAT
addressing (the zero-initialised sampler of src/scenes/model_render_scene.cpp:191-198).
Every per-sample operation is a float32 operation in the order the CUDA kernel uses; fused
multiply-adds are evaluated in float64 and rounded once.

density_grid(): sum_j m W(|x_node - x_j|) in float64 (CubicSpline, kernels_3d.slang:62-76).
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def _fma(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(f32)


def invert4(m):
    """Gauss-Jordan with partial pivoting on a column-major 4x4, in float64 (the host's order)."""
    a = np.zeros((4, 8))
    for r in range(4):
        for c in range(4):
            a[r, c] = m[4 * c + r]
        a[r, 4 + r] = 1.0
    for c in range(4):
        piv = c
        for r in range(c + 1, 4):
            if abs(a[r, c]) > abs(a[piv, c]):
                piv = r
        if a[piv, c] == 0.0:
            raise ValueError("singular")
        if piv != c:
            a[[c, piv]] = a[[piv, c]]
        inv = 1.0 / a[c, c]
        a[c] *= inv
        for r in range(4):
            if r != c and a[r, c] != 0.0:
                a[r] -= a[r, c] * a[c]
    out = np.zeros(16)
    for r in range(4):
        for c in range(4):
            out[4 * c + r] = a[r, 4 + c]
    return out


def mul4(a, b):
    out = np.zeros(16)
    for r in range(4):
        for c in range(4):
            s = 0.0
            for k in range(4):
                s += a[4 * k + r] * b[4 * c + k]
            out[4 * c + r] = s
    return out


def mac_style(x):
    """IDL Mac style (colormap.slang) on a float32 array; alpha is 1."""
    x = np.clip(x.astype(f32), f32(0), f32(1))
    h = (f32(-7.44992704834645e-01) * x).astype(f32) + f32(7.47986634976377e-01)
    i2 = np.fmod(np.fmod(x * f32(256), f32(2)) + f32(2), f32(2))
    v = np.where((i2 >= 0) & (i2 < 1), f32(1), f32(254.0 / 255.0)).astype(f32)
    h = (h * f32(6)).astype(f32)
    i = np.trunc(h).astype(np.int64)
    fr = (h - i.astype(f32)).astype(f32)
    f1 = (f32(1) - fr).astype(f32)
    f2 = (f32(1) - f1).astype(f32)
    z = np.zeros_like(v)
    r = np.select([i == 1, i == 2, i == 3, i == 4, i == 5], [v * f1, z, z, v * f2, v], v)
    g = np.select([i == 1, i == 2, i == 3, i == 4, i == 5], [v, v, v * f1, z, z], v * f2)
    b = np.select([i == 1, i == 2, i == 3, i == 4, i == 5], [z, v * f2, v, v, v * f1], z)
    return r.astype(f32), g.astype(f32), b.astype(f32)


def _sample(field, u, v, w):
    nz, ny, nx = field.shape
    tu = (u * f32(nx)).astype(f32) - f32(0.5)
    tv = (v * f32(ny)).astype(f32) - f32(0.5)
    tw = (w * f32(nz)).astype(f32) - f32(0.5)
    fu, fv, fw = np.floor(tu), np.floor(tv), np.floor(tw)
    au, av, aw = (tu - fu).astype(f32), (tv - fv).astype(f32), (tw - fw).astype(f32)
    i0, j0, k0 = fu.astype(np.int64), fv.astype(np.int64), fw.astype(np.int64)
    i1, j1, k1 = np.mod(i0 + 1, nx), np.mod(j0 + 1, ny), np.mod(k0 + 1, nz)
    i0, j0, k0 = np.mod(i0, nx), np.mod(j0, ny), np.mod(k0, nz)

    def lerp(a, b, t):
        return _fma(t, (b - a).astype(f32), a)

    c00 = lerp(field[k0, j0, i0], field[k0, j0, i1], au)
    c10 = lerp(field[k0, j1, i0], field[k0, j1, i1], au)
    c01 = lerp(field[k1, j0, i0], field[k1, j0, i1], au)
    c11 = lerp(field[k1, j1, i0], field[k1, j1, i1], au)
    return lerp(lerp(c00, c10, av), lerp(c01, c11, av), aw)


def raymarch(field, center, half, view, proj, width, height, step=0.05, n_steps=1000,
             color_scale=5.0, emission=200.0, background=None):
    field = np.asarray(field, f32)
    center = np.asarray(center, f32)
    half = np.asarray(half, f32)
    lo = (center - half).astype(f32)
    hi = (center + half).astype(f32)
    v64 = np.asarray(view, f32).astype(np.float64)
    p64 = np.asarray(proj, f32).astype(np.float64)
    ivp = invert4(mul4(p64, v64)).astype(f32)
    iv = invert4(v64)
    cam = np.array([iv[12] / iv[15], iv[13] / iv[15], iv[14] / iv[15]]).astype(f32)
    step, color_scale, emission = f32(step), f32(color_scale), f32(emission)

    px, py = np.meshgrid(np.arange(width), np.arange(height))
    ndx = (((f32(2) * px.astype(f32) + f32(1)) / f32(width)).astype(f32) - f32(1)).astype(f32)
    ndy = (((f32(2) * py.astype(f32) + f32(1)) / f32(height)).astype(f32) - f32(1)).astype(f32)

    def unproject(z):
        m = ivp
        X = m[0] * ndx + m[4] * ndy + m[8] * f32(z) + m[12]
        Y = m[1] * ndx + m[5] * ndy + m[9] * f32(z) + m[13]
        Z = m[2] * ndx + m[6] * ndy + m[10] * f32(z) + m[14]
        W = m[3] * ndx + m[7] * ndy + m[11] * f32(z) + m[15]
        return (X / W).astype(f32), (Y / W).astype(f32), (Z / W).astype(f32)

    ax_, ay_, az_ = unproject(0.0)
    bx_, by_, bz_ = unproject(1.0)
    d = [(bx_ - ax_).astype(f32), (by_ - ay_).astype(f32), (bz_ - az_).astype(f32)]
    il = (f32(1) / np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])).astype(f32)
    d = [(c * il).astype(f32) for c in d]
    t0 = np.full(d[0].shape, -np.inf, f32)
    t1 = np.full(d[0].shape, np.inf, f32)
    for k in range(3):
        nz = d[k] != 0
        with np.errstate(divide="ignore", invalid="ignore"):
            ta = ((lo[k] - cam[k]) / d[k]).astype(f32)
            tb = ((hi[k] - cam[k]) / d[k]).astype(f32)
        t0 = np.where(nz, np.maximum(t0, np.minimum(ta, tb)), t0)
        t1 = np.where(nz, np.minimum(t1, np.maximum(ta, tb)), t1)
        if cam[k] < lo[k] or cam[k] > hi[k]:
            t1 = np.where(nz, t1, -np.inf).astype(f32)
    hit = t1 >= np.maximum(t0, f32(0))
    tf = np.where(t0 > 0, t0, t1).astype(f32)
    tf = np.where(hit, tf, f32(0))
    pos = [_fma(tf, d[k], cam[k]) for k in range(3)]
    sd = [(d[k] * step).astype(f32) for k in range(3)]
    light = [np.zeros(d[0].shape, f32) for _ in range(4)]
    active = hit.copy()
    for s in range(n_steps):
        a = [((pos[k] - center[k]).astype(f32) / half[k]).astype(f32) for k in range(3)]
        if s == 0:
            a = [np.clip(ak, f32(-1), f32(1)) for ak in a]
        inside = np.ones_like(active)
        for k in range(3):
            inside &= (a[k] >= -1) & (a[k] <= 1)
        active &= inside
        if not active.any():
            break
        uvw = [(f32(0.5) * (a[k] + f32(1)).astype(f32)).astype(f32) for k in range(3)]
        dv = _sample(field, *uvw)
        r, g, b = mac_style((dv * color_scale).astype(f32))
        for ch, c in enumerate((r, g, b)):
            term = (step * ((c * dv).astype(f32) * emission).astype(f32)).astype(f32)
            light[ch] = np.where(active, (light[ch] + term).astype(f32), light[ch])
        term = (step * (dv * emission).astype(f32)).astype(f32)
        light[3] = np.where(active, (light[3] + term).astype(f32), light[3])
        pos = [np.where(active, (pos[k] + sd[k]).astype(f32), pos[k]) for k in range(3)]
    img = np.zeros((height, width, 4), f32) if background is None else np.array(background, f32) * np.ones((height, width, 4), f32)
    src = [np.clip(c, f32(0), f32(1)) for c in light]
    ia = (f32(1) - src[3]).astype(f32)
    out = img.copy()
    for ch in range(3):
        out[..., ch] = _fma(img[..., ch], ia, (src[ch] * src[3]).astype(f32))
    out[..., 3] = _fma(img[..., 3], ia, src[3])
    return np.where(hit[..., None], out, img)


def density_grid(pos, mass, h, lo, hi, res):
    """sum_j m W(|x - x_j|) at the grid nodes, float64; shape (res_z, res_y, res_x)."""
    pos = np.asarray(pos, np.float64)
    axes = []
    for a in range(3):
        n = int(res[a])
        axes.append(np.array([lo[a]], np.float64) if n == 1 else
                    lo[a] + np.arange(n) * ((hi[a] - lo[a]) / (n - 1)))
    zz, yy, xx = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    nodes = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1)
    sigma = 8.0 / (np.pi * h ** 3)
    out = np.zeros(len(nodes))
    for k in range(0, len(pos), 512):
        d = np.linalg.norm(nodes[:, None, :] - pos[None, k:k + 512, :], axis=2)
        q = d / h
        w = np.where(q <= 0.5, 6 * q ** 3 - 6 * q ** 2 + 1, np.where(q <= 1.0, 2 * (1 - q) ** 3, 0.0))
        out += mass * sigma * w.sum(1)
    return out.reshape(zz.shape)
