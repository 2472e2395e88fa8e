"""The README's usage example, run as written (files go to a temporary directory)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs

pytestmark = pytest.mark.gpu
SCENE = Path(__file__).resolve().parent / "golden" / "scenes" / "dam_break.json"


def test_readme_example(tmp_path):
    m = vfs.load_scene(str(SCENE))
    m.step()
    state = m.copy_data_buffers()
    keys, sorted_indices, offsets = m.get_neighbor_arrays()
    assert state["positions"].shape[0] == len(keys) == len(sorted_indices) == len(offsets)
    state = m.step_host(state["positions"], state["velocities"], substeps=1)
    assert np.isfinite(state["positions"]).all() and state["densities"].min() > 0.0

    view = vfs.look_at((12.0, -8.0, 9.0), (5.0, 5.0, 2.0))
    proj = vfs.perspective(0.8, 16 / 9, 0.1, 100.0)
    rgba = m.render_particles(view, proj, 1280, 720, quad_side=0.15)
    vfs.write_ppm(tmp_path / "particles.ppm", rgba)
    grid = m.density_grid((0, 0, 0), (10, 10, 8), (100, 100, 80)) / 1000.0
    img = vfs.render_density_raymarch(grid, (5, 5, 4), (5, 5, 4), view, proj, 1280, 720, step=0.05)
    vfs.write_ppm(tmp_path / "density.ppm", vfs.to_rgba8(img))
    assert (tmp_path / "particles.ppm").stat().st_size > 1280 * 720 * 3
    assert (tmp_path / "density.ppm").stat().st_size > 1280 * 720 * 3
    assert grid.max() > 0.5 and np.isfinite(img).all() and img[..., 3].max() > 0.0
