"""Triangle-mesh boundary objects: the oracle's mesh SDF restatement (CPU) and the GPU's mesh SDF
grid, volume map and signed-distance primitive against it."""
from __future__ import annotations

import json

import numpy as np
import pytest

from oracle import binding as ob
from tests import meshes

HALF = (0.3, 0.2, 0.25)


def _box_sdf(p, half):
    q = np.abs(np.asarray(p, np.float64)) - np.asarray(half)
    return np.linalg.norm(np.maximum(q, 0), axis=1) + np.minimum(q.max(1), 0)


def test_oracle_mesh_distance_of_a_box_is_the_box_sdf():
    v, t = meshes.box(HALF)
    p = np.random.default_rng(0).uniform(-0.6, 0.6, (3000, 3)).astype(np.float32)
    assert np.abs(ob.mesh_distance(v, t, p) - _box_sdf(p, HALF)).max() < 1e-7


def test_oracle_mesh_distance_signs_on_a_sphere():
    v, t = meshes.icosphere(0.3, 2)
    p = np.random.default_rng(1).uniform(-0.5, 0.5, (3000, 3)).astype(np.float32)
    d = ob.mesh_distance(v, t, p)
    r = np.linalg.norm(p.astype(np.float64), axis=1)
    clear = np.abs(r - 0.3) > 0.01  # the facets lie within 0.006 of the sphere
    assert (np.sign(d[clear]) == np.sign(r[clear] - 0.3)).all()
    assert np.abs(d - (r - 0.3)).max() < 0.01


def test_oracle_mesh_volume_map_of_a_box_equals_the_analytic_box():
    h = 0.04
    a = ob.mesh_volume_map(*meshes.box(HALF), h, (12, 12, 12), 8 * h)
    b = ob.volume_map(1, HALF, h, (12, 12, 12), 8 * h)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.abs(a[2] - b[2]).max() < 1e-6
    assert np.abs(a[3] - b[3]).max() <= 1e-6 * np.abs(b[3]).max()


def test_oracle_rejects_a_degenerate_mesh():
    v = np.zeros((3, 3), np.float32)
    with pytest.raises(ValueError):
        ob.mesh_distance(v, np.array([[0, 1, 2]]), np.zeros((1, 3)))


gpu = pytest.mark.gpu


@gpu
def test_gpu_signed_distance_matches_the_oracle():
    import vkfluidsim_gb300 as vfs

    v, t = meshes.icosphere(0.3, 2)
    p = np.random.default_rng(2).uniform(-0.6, 0.6, (5000, 3)).astype(np.float32)
    d = vfs.mesh_signed_distance(v, t, p)
    assert np.abs(d - ob.mesh_distance(v, t, p)).max() < 1e-9


def _model(h=0.04):
    from vkfluidsim_gb300 import workloads as W

    w = W.dam_break(dims=(4, 4, 4), map_res=0)
    from dataclasses import replace

    w.sim = replace(w.sim, smooth_radius=h)
    return W.build_model(w)


@gpu
def test_mesh_box_grids_equal_the_analytic_box_grids():
    import vkfluidsim_gb300 as vfs

    m = _model()
    m.add_mesh_object(vfs.MeshObject(vertices=meshes.box(HALF)[0], triangles=meshes.box(HALF)[1],
                                     resolution=(20, 18, 16)))
    m.add_analytic_object(vfs.AnalyticObject(vfs.SHAPE_BOX, HALF, resolution=(20, 18, 16)))
    a, b = m.get_boundary_object(0), m.get_boundary_object(1)
    assert np.array_equal(a.box_pos, b.box_pos) and np.array_equal(a.box_size, b.box_size)
    assert np.abs(a.sdf - b.sdf).max() < 1e-6
    assert np.abs(a.volume_map - b.volume_map).max() <= 2e-6 * np.abs(b.volume_map).max()


@gpu
def test_mesh_grids_match_the_oracle():
    import vkfluidsim_gb300 as vfs

    v, t = meshes.icosphere(0.25, 1)
    h = 0.04
    m = _model(h)
    m.add_mesh_object(vfs.MeshObject(vertices=v, triangles=t, resolution=(16, 16, 16)))
    g = m.get_boundary_object(0)
    bs, bp, sdf, vm = ob.mesh_volume_map(v, t, h, (16, 16, 16), np.float32(8 * h))
    assert np.array_equal(g.box_size, bs) and np.array_equal(g.box_pos, bp)
    assert np.abs(g.sdf - sdf).max() < 1e-6
    assert np.abs(g.volume_map - vm).max() <= 1e-5 * np.abs(vm).max()


@gpu
def test_obj_file_object_equals_array_object(tmp_path):
    import vkfluidsim_gb300 as vfs

    v, t = meshes.icosphere(0.2, 1)
    meshes.write_obj(tmp_path / "s.obj", v, t, extra_object_first=True)
    m = _model()
    m.add_mesh_object(vfs.MeshObject(obj_path=str(tmp_path / "s.obj"), position=(0.5, 0.5, 0.3),
                                     resolution=(12, 12, 12)))
    m.add_mesh_object(vfs.MeshObject(vertices=v, triangles=t, position=(0.5, 0.5, 0.3),
                                     resolution=(12, 12, 12)))
    a, b = m.get_boundary_object(0), m.get_boundary_object(1)
    assert np.array_equal(a.sdf, b.sdf) and np.array_equal(a.volume_map, b.volume_map)
    assert np.array_equal(a.transform, b.transform)


@gpu
def test_scene_with_an_obj_boundary_object_loads_and_steps(tmp_path):
    import vkfluidsim_gb300 as vfs

    v, t = meshes.icosphere(0.15, 1)
    (tmp_path / "models").mkdir()
    meshes.write_obj(tmp_path / "models" / "ball.obj", v, t)
    scene = {
        "name": "mesh obstacle",
        "fluidModel": "wcsph",
        "wcsphParameters": {"stiffness": 50.0, "expoent": 7.0, "viscosityStrenght": 0.01,
                            "outerWallStiffness": 10000.0},
        "simulationParameters": {"gravity": [0.0, 0.0, -9.81], "smoothRadius": 0.04,
                                 "timeScale": 1.0, "iterations": 1, "dt": 2e-4,
                                 "targetDensity": 1000.0,
                                 "boundingBox": {"pos": [0, 0, 0], "size": [1, 1, 1]}},
        "fluidBlocks": [{"size": [12, 12, 12], "pos": [0.05, 0.05, 0.05]}],
        "boundaryObjects": [{"resourcePath": "models/ball.obj", "position": [0.6, 0.6, 0.2],
                             "rotation": {"angle": -90.0, "axis": [0, 1, 0]},
                             "scale": [1.0, 1.0, 0.5],
                             "volumeMapResolution": [16, 16, 16]}],
    }
    (tmp_path / "scene.json").write_text(json.dumps(scene))
    m = vfs.load_scene(str(tmp_path / "scene.json"), str(tmp_path))
    assert m.n_boundary_objects == 1
    m.substeps(10)
    assert np.isfinite(m.copy_data_buffers()["positions"]).all()


@gpu
def test_reference_obstacle_scene_loads_with_generated_meshes(tmp_path):
    """The reference's obstacle.json fixture, with its models/box.obj and models/suzanne.obj
    replaced by generated meshes (a unit box and an icosphere)."""
    import shutil

    import vkfluidsim_gb300 as vfs

    (tmp_path / "models").mkdir()
    meshes.write_obj(tmp_path / "models" / "box.obj", *meshes.box((0.5, 0.5, 0.5)))
    meshes.write_obj(tmp_path / "models" / "suzanne.obj", *meshes.icosphere(0.8, 1))
    src = __import__("pathlib").Path(__file__).parent / "golden" / "scenes" / "obstacle.json"
    shutil.copy(src, tmp_path / "obstacle.json")
    m = vfs.load_scene(str(tmp_path / "obstacle.json"), str(tmp_path))
    assert m.n_boundary_objects == 2
    for k in range(2):
        g = m.get_boundary_object(k)
        assert tuple(g.resolution) == (30, 30, 30)
        assert (g.sdf < 0).any() and (g.volume_map > 0).any()
    m.substeps(2)
    assert np.isfinite(m.copy_data_buffers()["positions"]).all()
