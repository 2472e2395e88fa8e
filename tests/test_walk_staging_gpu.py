"""The density walk's block-per-cell staging (a warp whose particles share a row of cells stages
the 3 x 3 rows around it in shared memory) must reproduce the per-thread bucket walk bit for bit:
same in-range neighbours, same visiting order, same sums and lists. Each case runs the same scene
with staging on and off and compares every output of every substep."""
from __future__ import annotations

import numpy as np
import pytest

from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _outputs(m):
    k, p, o = m.get_neighbor_arrays()
    s = m.copy_data_buffers()
    return [k, p, o, s["positions"], s["velocities"], s["densities"]]


def _same(a, b, label):
    for x, y in zip(a, b):
        assert np.array_equal(x, y), label


@pytest.mark.parametrize("skin", [0.0, 0.05])
def test_staging_is_bit_identical_on_the_1m_scene(skin):
    w = W.obstacle_1m()
    on, off = W.build_model(w), W.build_model(w)
    off.set_walk_staging(False)
    for m in (on, off):
        m.set_skin(skin)
    for s in range(4):
        on.substeps(1)
        off.substeps(1)
        _same(_outputs(on), _outputs(off), f"1M skin {skin} substep {s + 1}")


def test_staging_is_bit_identical_on_a_dam_break_and_a_batch():
    w = W.dam_break(dims=(40, 40, 40), map_res=32, stiffness=200.0)
    on, off = W.build_model(w), W.build_model(w)
    off.set_walk_staging(False)
    on.substeps(6)
    off.substeps(6)
    _same(_outputs(on), _outputs(off), "dam break")
    scenes = W.batched_scenes(n_scenes=24, n_min=20000, n_max=65536, map_res=24, seed=8)
    bon, boff = W.build_batch(scenes), W.build_batch(scenes)
    boff.set_walk_staging(False)
    bon.substeps(4)
    boff.substeps(4)
    for s in range(len(scenes)):
        a = list(bon.get_neighbor_arrays(s)) + list(bon.copy_data_buffers(s).values())
        b = list(boff.get_neighbor_arrays(s)) + list(boff.copy_data_buffers(s).values())
        _same(a, b, f"batch scene {s}")


@pytest.mark.parametrize("skin", [0.0, 0.05])
def test_staging_is_bit_identical_on_a_batch_with_small_scenes(skin):
    """Scenes of 2048 to 65,536 particles, so that list blocks and the last warp straddle scenes
    whose tables are too small to stage (n <= 5110) and scenes that stage: an idle lane holding a
    slot of another scene must not change the warp's choice or the rows it stages."""
    scenes = W.batched_scenes(n_scenes=48, n_min=2048, n_max=65536, map_res=24, seed=3)
    assert min(w.n for w in scenes) <= 5110 < max(w.n for w in scenes)
    bon, boff = W.build_batch(scenes), W.build_batch(scenes)
    boff.set_walk_staging(False)
    for b in (bon, boff):
        b.set_skin(skin)
        b.substeps(5)
    for s in range(len(scenes)):
        a = list(bon.get_neighbor_arrays(s)) + list(bon.copy_data_buffers(s).values())
        b = list(boff.get_neighbor_arrays(s)) + list(boff.copy_data_buffers(s).values())
        _same(a, b, f"batch scene {s} (skin {skin})")


def test_staging_is_bit_identical_on_the_stress_workload():
    w = W.stress_4m()
    on, off = W.build_model(w), W.build_model(w)
    off.set_walk_staging(False)
    for m in (on, off):
        m.set_neighbor_capacity(1536)
        m.substeps(1)
    _same(_outputs(on), _outputs(off), "stress")
