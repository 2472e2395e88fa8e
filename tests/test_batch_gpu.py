"""GPU tests of batched scenes: one vfs_batch advancing many independent scenes must give, for every
scene, the neighbour arrays (bit-exact) and fields of that scene run alone (tests/helpers.py
tolerances), and agree with the oracle."""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from tests.helpers import RTOL, normwise_rel
from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _mixed_scenes():
    """Uneven scenes: a tiny table with colliding keys, plain lattices, a sphere obstacle,
    different parameters per scene."""
    scenes = W.batched_scenes(n_scenes=5, n_min=300, n_max=20000, map_res=24, seed=9)
    tiny = W.dam_break(dims=(2, 2, 2), map_res=0)
    rng = np.random.default_rng(4)
    tiny.pos = (rng.random((37, 3)) * 0.12).astype(np.float32)
    tiny.vel = ((rng.random((37, 3)) - 0.5) * 0.1).astype(np.float32)
    tiny.sph = replace(tiny.sph, n_particles=37)
    sphere = W.dam_break(dims=(20, 20, 12), spacing=0.02, map_res=0, stiffness=100.0, seed=5)
    sphere.objects = [vfs.AnalyticObject(vfs.SHAPE_SPHERE, (0.1,), position=(0.3, 0.3, 0.1),
                                         resolution=(32, 32, 32))]
    sphere.vel = ((rng.random(sphere.pos.shape) - 0.5) * 0.3).astype(np.float32)
    return [scenes[0], tiny, scenes[1], sphere, scenes[2], scenes[3], scenes[4]]


def test_batch_equals_each_scene_alone():
    scenes = _mixed_scenes()
    b = W.build_batch(scenes)
    b.record_fields(True)
    b.substeps(3)
    for s, w in enumerate(scenes):
        m = W.build_model(w)
        m.record_fields(True)
        m.substeps(3)
        bk, bp, bo = b.get_neighbor_arrays(s)
        mk, mp, mo = m.get_neighbor_arrays()
        assert np.array_equal(bk, mk) and np.array_equal(bp, mp) and np.array_equal(bo, mo), s
        assert np.array_equal(b.get_ids(s), m.get_ids())
        gb, gm = b.copy_data_buffers(s, with_acc=True), m.copy_data_buffers(with_acc=True)
        for k in gm:
            assert normwise_rel(gb[k], gm[k]) <= RTOL, (s, k)


def test_batch_scene_against_the_oracle():
    from tests.helpers import oracle_for

    scenes = _mixed_scenes()
    b = W.build_batch(scenes)
    b.substeps(1)
    for s in (1, 3, 5):
        w = scenes[s]
        m = W.build_model(w)  # the oracle takes the same boundary grids
        o = oracle_for(w, m)
        o.substeps(1)
        ok, op, oo = o.neighbors()
        bk, bp, bo = b.get_neighbor_arrays(s)
        assert np.array_equal(bk, ok) and np.array_equal(bp, op) and np.array_equal(bo, oo)
        g, r = b.copy_data_buffers(s), o.state()
        for k in ("positions", "velocities", "densities"):
            assert normwise_rel(g[k], r[k]) <= RTOL, (s, k)


def test_many_small_scenes_with_graph_and_parameter_update():
    scenes = W.batched_scenes(n_scenes=64, n_min=64, n_max=3000, map_res=16, seed=21)
    b = W.build_batch(scenes)
    b.substeps(2)
    # Changing one scene's viscosity re-captures the graph and affects only that scene.
    w5 = scenes[5]
    b.set_scene_parameters(5, wcsph=replace(w5.wcsph, viscosity_strenght=0.2))
    b.substeps(2)
    for s in (0, 5, 17, 63):
        w = scenes[s]
        m = W.build_model(w)
        m.substeps(2)
        if s == 5:
            m.set_parameters(wcsph=replace(w5.wcsph, viscosity_strenght=0.2))
        m.substeps(2)
        assert np.array_equal(b.get_neighbor_arrays(s)[1], m.get_neighbor_arrays()[1])
        gb, gm = b.copy_data_buffers(s), m.copy_data_buffers()
        for k in gm:
            assert normwise_rel(gb[k], gm[k]) <= RTOL, (s, k)
    b.synchronize()
