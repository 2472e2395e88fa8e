"""Density raymarch (raymarch.slang) and the density grid against the NumPy restatement in
tests/raymarch_reference.py, plus known answers that pin the semantics: fixed steps from the
visible face of the field's box, REPEAT sampling, the [0, 1] clamp and the alpha blend."""
from __future__ import annotations

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from tests import raymarch_reference as R
from vkfluidsim_gb300 import workloads as W

gpu = pytest.mark.gpu


def camera(eye, target, up, width, height):
    view = vfs.look_at(eye, target, up)
    proj = vfs.perspective(np.deg2rad(50.0), width / height, 0.05, 20.0)
    return view, proj


def blob_field(shape, seed=0):
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.linspace(-1, 1, nz), np.linspace(-1, 1, ny), np.linspace(-1, 1, nx),
                          indexing="ij")
    f = np.exp(-3.0 * (x * x + 1.5 * y * y + 2.0 * z * z)) + 0.05 * rng.random(shape)
    return f.astype(np.float32)


def constant_case(c0=0.1):
    field = np.full((8, 8, 8), c0, np.float32)
    center, half = np.array([0.3, -0.2, 0.1]), np.array([0.4, 0.5, 0.5])
    return field, center, half


def expected_from_samples(n, c0, step, cs, em, bg):
    r, g, b = R.mac_style(np.array([np.float32(c0) * np.float32(cs)], np.float32))
    light = []
    for c in (r[0], g[0], b[0], np.float32(1.0)):
        acc = np.float32(0)
        term = np.float32(step) * (np.float32(c * np.float32(c0)) * np.float32(em))
        for _ in range(n):
            acc = np.float32(acc + term)
        light.append(min(max(float(acc), 0.0), 1.0))
    sa = light[3]
    return np.array([light[0] * sa + bg[0] * (1 - sa), light[1] * sa + bg[1] * (1 - sa),
                     light[2] * sa + bg[2] * (1 - sa), sa + bg[3] * (1 - sa)])


def test_oracle_known_answer_outside_and_inside():
    """The restatement itself: 34 samples straight through the box, 1 from inside."""
    field, center, half = constant_case()
    bg = np.array([0.2, 0.3, 0.4, 1.0], np.float32)
    view, proj = camera((0.3, -0.2, 2.0), (0.3, -0.2, 0.1), (0, 1, 0), 33, 33)
    img = R.raymarch(field, center, half, view, proj, 33, 33, step=0.03, n_steps=1000,
                     color_scale=5.0, emission=0.2, background=bg)
    np.testing.assert_allclose(img[16, 16], expected_from_samples(34, 0.1, 0.03, 5.0, 0.2, bg),
                               rtol=1e-5)
    view, proj = camera((0.3, -0.2, 0.2), (0.3, -0.2, -0.3), (0, 1, 0), 33, 33)
    img = R.raymarch(field, center, half, view, proj, 33, 33, step=0.03, n_steps=1000,
                     color_scale=5.0, emission=0.2, background=bg)
    np.testing.assert_allclose(img[16, 16], expected_from_samples(1, 0.1, 0.03, 5.0, 0.2, bg),
                               rtol=1e-5)


@gpu
def test_raymarch_known_answers():
    field, center, half = constant_case()
    bg = np.array([0.2, 0.3, 0.4, 1.0], np.float32)
    for eye, target, n in (((0.3, -0.2, 2.0), (0.3, -0.2, 0.1), 34),  # through the box
                           ((0.3, -0.2, 0.2), (0.3, -0.2, -0.3), 1)):  # from inside: exit face
        view, proj = camera(eye, target, (0, 1, 0), 33, 33)
        img = vfs.render_density_raymarch(field, center, half, view, proj, 33, 33, step=0.03,
                                          color_scale=5.0, emission=0.2, background=bg)
        np.testing.assert_allclose(img[16, 16], expected_from_samples(n, 0.1, 0.03, 5.0, 0.2, bg),
                                   rtol=1e-5)
    # A pixel whose ray misses the box keeps the background.
    view, proj = camera((0.3, -0.2, 2.0), (0.3, -0.2, 0.1), (0, 1, 0), 33, 33)
    img = vfs.render_density_raymarch(field, center, half, view, proj, 33, 33, step=0.03,
                                      emission=0.2, background=bg)
    np.testing.assert_array_equal(img[0, 0], bg)
    # Saturation: the reference's emission 200 clamps alpha to 1 in one step.
    img = vfs.render_density_raymarch(field, center, half, view, proj, 33, 33, background=bg)
    assert img[16, 16, 3] == 1.0


@gpu
@pytest.mark.parametrize("seed", [0, 1])
def test_raymarch_matches_restatement(seed):
    field = blob_field((10, 12, 14), seed)
    center, half = np.array([0.1, 0.2, -0.1]), np.array([0.7, 0.5, 0.4])
    eyes = [(1.8, -1.4, 1.1), (-0.9, 1.6, -1.2)]
    view, proj = camera(eyes[seed], center, (0, 0, 1), 48, 40)
    bg = np.array([0.05, 0.1, 0.15, 0.5], np.float32)
    kw = dict(step=0.02, n_steps=1000, color_scale=5.0, emission=3.0, background=bg)
    got = vfs.render_density_raymarch(field, center, half, view, proj, 48, 40, **kw)
    ref = R.raymarch(field, center, half, view, proj, 48, 40, **kw)
    err = np.abs(got - ref)
    # Ray set-up rounding (fused multiply-adds on the device) moves samples by ~1 ulp; the colour
    # map's 1/255 value steps and the last sample at the exit face are the only jumps.
    assert err.max() <= 5e-3, err.max()
    assert err.mean() <= 2e-5, err.mean()
    assert (got[..., 3] > 0.01).sum() > 200  # the blob is visible


@gpu
def test_raymarch_device_buffers_match_host():
    torch = pytest.importorskip("torch")
    field = blob_field((9, 11, 13), 3)
    center, half = np.zeros(3), np.array([0.5, 0.6, 0.7])
    view, proj = camera((1.5, 1.2, 0.9), center, (0, 0, 1), 40, 30)
    host = vfs.render_density_raymarch(field, center, half, view, proj, 40, 30, step=0.02,
                                       emission=3.0)
    import ctypes as C

    from vkfluidsim_gb300._abi import check

    fd = torch.from_numpy(field).cuda()
    img = torch.zeros((30, 40, 4), dtype=torch.float32, device="cuda")
    res = np.array([13, 11, 9], np.int32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    tp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_float))  # noqa: E731
    c, h = np.asarray(center, np.float32), np.asarray(half, np.float32)
    check(vfs.load_library().vfs_render_density_raymarch(
        tp(fd), res.ctypes.data_as(C.POINTER(C.c_int32)), fp(c), fp(h), fp(view), fp(proj), 40, 30,
        0.02, 1000, 5.0, 3.0, tp(img)))
    np.testing.assert_array_equal(img.cpu().numpy(), host)


@gpu
def test_density_grid_matches_restatement():
    w = W.dam_break(dims=(10, 10, 10), spacing=0.02, box=(0.5, 0.5, 0.5), map_res=16, seed=2)
    m = W.build_model(w)
    m.substeps(2)
    st = m.copy_data_buffers()
    lo, hi, res = (-0.02, -0.02, -0.02), (0.24, 0.22, 0.25), (11, 10, 9)
    got = m.density_grid(lo, hi, res)
    mass = w.sph.target_density * 0.8 * w.sim.smooth_radius ** 3 / 8.0
    ref = R.density_grid(st["positions"], mass, w.sim.smooth_radius, lo, hi, res)
    assert got.shape == (9, 10, 11)
    assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref)
    # A grid of one node per axis sits at lo.
    one = m.density_grid(st["positions"][0], st["positions"][0], (1, 1, 1))
    ref1 = R.density_grid(st["positions"], mass, w.sim.smooth_radius, st["positions"][0],
                          st["positions"][0], (1, 1, 1))
    np.testing.assert_allclose(one, ref1, rtol=1e-5)


@gpu
def test_density_grid_batch_scene_and_raymarch():
    scenes = [W.dam_break(dims=(8, 8, 8), spacing=0.02, box=(0.4, 0.4, 0.4), map_res=16, seed=s)
              for s in range(2)]
    b = W.build_batch(scenes)
    b.substeps(1)
    st = b.copy_data_buffers(1)
    lo, hi, res = (0.0, 0.0, 0.0), (0.16, 0.16, 0.16), (8, 8, 8)
    got = b.density_grid(1, lo, hi, res)
    mass = scenes[1].sph.target_density * 0.8 * scenes[1].sim.smooth_radius ** 3 / 8.0
    ref = R.density_grid(st["positions"], mass, scenes[1].sim.smooth_radius, lo, hi, res)
    assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref)
    # The field, normalised by rho0, rendered with the reference's constants.
    view, proj = camera((0.6, -0.4, 0.5), (0.08, 0.08, 0.08), (0, 0, 1), 32, 32)
    img = vfs.render_density_raymarch(got / 1000.0, (0.08, 0.08, 0.08), (0.08, 0.08, 0.08), view,
                                      proj, 32, 32)
    assert np.isfinite(img).all() and img[..., 3].max() == 1.0
    assert vfs.to_rgba8(img).dtype == np.uint8
