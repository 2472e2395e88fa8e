"""Headless particle rendering on the GPU against the NumPy restatement (tests/render_reference.py)
and an analytic single-particle case."""
from __future__ import annotations

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from tests import render_reference as RR
from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _model(pos, vel):
    w = W.dam_break(dims=(2, 2, 2), map_res=0)
    w.pos, w.vel = np.asarray(pos, np.float32), np.asarray(vel, np.float32)
    return W.build_model(w)


def test_single_particle_disc():
    m = _model([[0.5, 0.5, 0.5]], [[0.0, 0.0, 0.0]])
    mv = vfs.look_at((0.5, 0.5, 2.5), (0.5, 0.5, 0.5), (0.0, 1.0, 0.0))
    pj = vfs.perspective(0.8, 1.0, 0.1, 10.0)
    img, dep = m.render_particles(mv, pj, 256, 256, with_depth=True)
    ref, _ = RR.render(np.array([[0.5, 0.5, 0.5]]), np.zeros((1, 3)), mv, pj, 256, 256)
    # Near the centre n ~ (0, 0, 1): diffuse ~ 1/sqrt(2) of the colour map at 0 = (0.4880, 0, 1).
    c = img[127:129, 127:129, :3].astype(int)
    assert np.abs(c - ref[127:129, 127:129, :3].astype(int)).max() <= 2
    assert np.abs(c - np.round(RR.mac_style(0.0) / np.sqrt(2.0) * 255)).max() <= 12
    covered = dep < 1.0
    # Radius in pixels: half side 0.075 at distance 2 with f = 1/tan(0.4), 128 px per NDC unit.
    r_px = 0.075 / 2.0 / np.tan(0.4) * 128
    assert abs(np.sqrt(covered.sum() / np.pi) - r_px) < 1.0
    assert (img[~covered][:, :3] == 0).all() and (img[..., 3] == 255).all()


def test_matches_numpy_restatement():
    rng = np.random.default_rng(3)
    n = 40
    pos = rng.uniform(0.2, 0.8, (n, 3))
    vel = rng.normal(0.0, 3.0, (n, 3))
    m = _model(pos, vel)
    mv = vfs.look_at((1.8, -1.2, 1.4), (0.5, 0.5, 0.5))
    pj = vfs.perspective(0.9, 1.25, 0.05, 20.0)
    img = m.render_particles(mv, pj, 80, 64, quad_side=0.3, depth_radius=0.15, v_max=6.5)
    # The model holds the particles in its own order: restate with the same order.
    s = m.copy_data_buffers()
    ref, owner = RR.render(s["positions"].astype(np.float64), s["velocities"].astype(np.float64),
                           mv, pj, 80, 64, quad_side=0.3, depth_radius=0.15)
    cov_gpu = img[..., :3].sum(-1) > 0
    cov_ref = ref[..., :3].sum(-1) > 0
    assert (cov_gpu != cov_ref).mean() < 0.01  # disc edges may round differently
    both = cov_gpu & cov_ref
    assert both.sum() > 200
    diff = np.abs(img[both][:, :3].astype(int) - ref[both][:, :3].astype(int)).max(axis=1)
    assert (diff <= 2).mean() > 0.98  # a pixel whose winner flips on a depth tie may differ


def test_offscreen_and_behind_camera_particles_draw_nothing():
    m = _model([[0.5, 0.5, 5.0], [50.0, 0.5, 0.5]], [[0, 0, 0], [0, 0, 0]])
    mv = vfs.look_at((0.5, 0.5, 2.5), (0.5, 0.5, 0.5), (0.0, 1.0, 0.0))
    pj = vfs.perspective(0.8, 1.0, 0.1, 10.0)
    img = m.render_particles(mv, pj, 32, 32)
    assert (img[..., :3] == 0).all()


def test_writes_a_ppm(tmp_path):
    w = W.dam_break(dims=(16, 16, 16), map_res=0)
    m = W.build_model(w)
    m.substeps(2)
    img = m.render_particles(vfs.look_at((1.5, -1.0, 1.2), (0.15, 0.15, 0.15)),
                             vfs.perspective(0.7, 4 / 3, 0.05, 20.0), 160, 120, quad_side=0.02)
    vfs.write_ppm(tmp_path / "f.ppm", img)
    data = (tmp_path / "f.ppm").read_bytes()
    assert data.startswith(b"P6\n160 120\n255\n") and len(data) == 15 + 160 * 120 * 3
    assert (img[..., :3].sum(-1) > 0).mean() > 0.01
