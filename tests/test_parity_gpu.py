"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle on identical inputs.

Bars: sort keys, sorted_indices (permutation) and spatial offsets bit-exact; boundary terms,
densities, accelerations, velocities and positions within RTOL = 1e-5 normwise relative error
(tests/helpers.py); the FP32-vs-FP64 error of the same step is printed beside it.
"""
from __future__ import annotations

import json
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from tests.helpers import RTOL, by_id, compare_step, normwise_rel, oracle_for
from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
M32 = np.uint64(0xFFFFFFFF)


def np_keys(pos, h, n):
    """Vectorised HashCell3D(floor(x / h)) % n (spatial_hash_3d.slang:16-32)."""
    c = np.floor(pos.astype(np.float32) / np.float32(h)).astype(np.int64)
    u = (c + 25) & 0xFFFFFFFF
    loc, blk = u % 50, u // 50
    bh = (blk[:, 0] * 15823 + blk[:, 1] * 9737333 + blk[:, 2] * 440817757) & 0xFFFFFFFF
    hsh = (loc[:, 0] + 50 * (loc[:, 1] + 50 * loc[:, 2]) + bh) & 0xFFFFFFFF
    return (hsh % n).astype(np.uint32)


@pytest.fixture(scope="module")
def dam():
    w = W.dam_break(dims=(24, 24, 24), map_res=32, stiffness=200.0)
    w.pos[:, 2] -= 0.005  # some particles start below the floor: wall penalty is exercised
    return w


def test_first_substep_parity_dam_break(dam):
    m = W.build_model(dam)
    o = oracle_for(dam, m)
    o64 = oracle_for(dam, m, fp64=True)
    errs = compare_step(m, o, "dam_break_13824", fp64_oracle=o64)
    bd, _ = m.get_boundary_fields()
    assert (bd > 0).sum() > 100, "the volume map must contribute"
    # The GPU's FP32 error against FP64 stays at the oracle's own FP32 error level.
    for k in ("densities", "velocities", "positions"):
        assert errs[f"gpu_vs_fp64_{k}"] <= max(4 * errs[f"oracle32_vs_fp64_{k}"], 1e-6)


def test_per_step_parity_from_identical_state(dam):
    """Advance 40 substeps on the GPU, load that state into the oracle, compare one substep."""
    m = W.build_model(dam)
    m.substeps(40)
    s = m.copy_data_buffers()
    ids = m.get_ids()
    o = oracle_for(dam, m, pos=s["positions"], vel=s["velocities"], ids=ids)
    errs = compare_step(m, o, "dam_break_after_40")
    assert np.abs(s["velocities"]).max() > 1e-3


def test_multistep_drift_is_bounded():
    w = W.dam_break(dims=(16, 16, 16), map_res=24, stiffness=200.0)
    m = W.build_model(w)
    o = oracle_for(w, m)
    m.substeps(200)
    o.substeps(200)
    g, r = m.copy_data_buffers(), o.state()
    gi, ri = m.get_ids(), r["ids"]
    drift = np.abs(by_id(g["positions"], gi) - by_id(r["positions"], ri)).max()
    travel = np.abs(by_id(g["positions"], gi) - w.pos).max()
    print("drift after 200 substeps:", drift, "max travel:", travel)
    assert travel > 1e-3
    assert drift < 1e-4


def test_sphere_obstacle_rotated_and_scaled():
    w = W.dam_break(dims=(20, 20, 12), spacing=0.02, map_res=0, stiffness=100.0)
    rng = np.random.default_rng(11)
    w.pos[:] = (rng.random(w.pos.shape) * (0.6, 0.6, 0.4) + (0.1, 0.1, 0.0)).astype(np.float32)
    w.vel[:] = ((rng.random(w.vel.shape) - 0.5) * 0.5).astype(np.float32)
    w.objects = [
        vfs.AnalyticObject(vfs.SHAPE_SPHERE, (0.12,), position=(0.4, 0.4, 0.15),
                           rotation_angle_deg=30.0, rotation_axis=(1.0, 1.0, 0.0),
                           scale=(1.0, 1.0, 1.0), resolution=(40, 40, 40)),
        vfs.AnalyticObject(vfs.SHAPE_BOX, (0.1, 0.05, 0.08), position=(0.2, 0.6, 0.1),
                           rotation_angle_deg=-90.0, rotation_axis=(0.0, 1.0, 0.0),
                           scale=(1.0, 2.0, 1.0), resolution=(24, 24, 24)),
    ]
    m = W.build_model(w)
    o = oracle_for(w, m)
    compare_step(m, o, "two_objects")
    bd, _ = m.get_boundary_fields()
    assert (bd > 0).sum() > 20


@pytest.mark.parametrize("n", [29, 57])
def test_tiny_tables_with_colliding_keys(n):
    w = W.dam_break(dims=(2, 2, 2), map_res=0)
    rng = np.random.default_rng(n)
    pos = (rng.random((n, 3)) * 0.12).astype(np.float32)
    w.pos, w.vel = pos, ((rng.random((n, 3)) - 0.5) * 0.1).astype(np.float32)
    w.sph = replace(w.sph, n_particles=n)
    m = W.build_model(w)
    o = oracle_for(w, m)
    for _ in range(3):
        compare_step(m, o, f"tiny_{n}")


@pytest.mark.parametrize("n", [0, 1, 2, 255, 4097])
def test_edge_sizes(n):
    w = W.dam_break(dims=(2, 2, 2), map_res=0)
    rng = np.random.default_rng(100 + n)
    w.pos = (rng.random((n, 3)) * 0.3).astype(np.float32)
    w.vel = np.zeros((n, 3), np.float32)
    w.sph = replace(w.sph, n_particles=n)
    m = W.build_model(w)
    if n == 0:
        m.substeps(2)
        m.synchronize()
        assert m.copy_data_buffers()["positions"].shape == (0, 3)
        return
    o = oracle_for(w, m)
    compare_step(m, o, f"n={n}")


@pytest.mark.parametrize("digits,items", [(4, 8), (5, 12), (6, 16), (7, 8), (8, 12), (8, 16)])
def test_sort_configurations_are_bit_exact(digits, items):
    w = W.stress_4m(n_uniform=60000, n_blob=9000, map_res=0)
    rng = np.random.default_rng(digits * 31 + items)
    w.pos = w.pos[rng.permutation(w.n)]
    m = W.build_model(w)
    m.set_sort_config(digits, items)
    o = oracle_for(w, m)
    compare_step(m, o, f"sort_{digits}_{items}", check_fields=False)


def test_graph_and_stream_launch_agree_bitwise(dam):
    a, b = W.build_model(dam), W.build_model(dam)
    b.use_graph(False)
    a.substeps(5)
    b.substeps(5)
    sa, sb = a.copy_data_buffers(), b.copy_data_buffers()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def test_full_size_one_million_particles():
    """The plain 1M workload at full size: 1,048,576 particles with the sphere map."""
    w = W.obstacle_1m(map_res=128)
    m = W.build_model(w)
    m.substeps(1)
    keys, perm, offs = m.get_neighbor_arrays()
    expected = np_keys(w.pos, w.sim.smooth_radius, w.n)
    assert np.array_equal(np.sort(perm), np.arange(w.n, dtype=np.uint32))
    assert np.array_equal(keys, expected[perm])
    same = keys[1:] == keys[:-1]
    assert np.all(np.diff(keys.astype(np.int64)) >= 0) and np.all(perm[1:][same] > perm[:-1][same])
    first = np.searchsorted(keys, np.arange(w.n, dtype=np.uint32))
    present = np.zeros(w.n, bool)
    present[keys] = True
    assert np.array_equal(offs, np.where(present, first, w.n).astype(np.uint32))
    # Full parity of one substep from that identical state.
    s = m.copy_data_buffers()
    o = oracle_for(w, m, pos=s["positions"], vel=s["velocities"], ids=m.get_ids())
    compare_step(m, o, "obstacle_1m")


@pytest.mark.parametrize("slots", [128, 1536])
def test_full_size_stress_workload(slots):
    """The stress workload at full size: 4,194,304 uniform particles in a 4 x 2 x 2 box plus a
    419,430-particle Gaussian blob (sigma 0.1, ~900 neighbours per particle), h = 0.02, 128^3
    container map. With 128 list slots the blob's lists overflow and the force pass walks the
    candidates; with 1,536 (the measured configuration) every list fits."""
    w = W.stress_4m()
    assert w.n == 4_613_734
    m = W.build_model(w)
    m.set_neighbor_capacity(slots)
    m.substeps(1)
    keys, perm, offs = m.get_neighbor_arrays()
    expected = np_keys(w.pos, w.sim.smooth_radius, w.n)
    assert np.array_equal(np.sort(perm), np.arange(w.n, dtype=np.uint32))
    assert np.array_equal(keys, expected[perm])
    same = keys[1:] == keys[:-1]
    assert np.all(np.diff(keys.astype(np.int64)) >= 0) and np.all(perm[1:][same] > perm[:-1][same])
    s = m.copy_data_buffers()
    o = oracle_for(w, m, pos=s["positions"], vel=s["velocities"], ids=m.get_ids())
    compare_step(m, o, f"stress_4m_{slots}_slots")
    g = m.copy_data_buffers()
    assert g["densities"].max() > 10 * np.median(g["densities"])


def test_volume_map_generation_matches_oracle():
    from oracle import binding as ob

    h = 0.015
    for shape, prm, res in ((vfs.SHAPE_SPHERE, (0.2,), (48, 48, 48)),
                            (vfs.SHAPE_CONTAINER, (0.5, 0.25, 0.25), (40, 24, 24)),
                            (vfs.SHAPE_BOX, (0.1, 0.2, 0.05), (20, 30, 16))):
        w = W.dam_break(dims=(2, 2, 2), map_res=0)
        w.sim = replace(w.sim, smooth_radius=h)
        w.objects = [vfs.AnalyticObject(shape, prm, resolution=res)]
        m = W.build_model(w)
        info = m.get_boundary_object(0)
        bs, bp, sdf, vm = ob.volume_map(shape, prm, h, res, np.float32(8.0 * h))
        assert np.array_equal(info.box_size, bs) and np.array_equal(info.box_pos, bp)
        assert np.array_equal(info.sdf, sdf)
        assert normwise_rel(info.volume_map, vm) < 1e-6
        assert (vm > 0).sum() > 100


def test_reference_dam_break_scene():
    """The reference's assets/scenes/dam_break.json: 75,000 particles, 3 iterations per step."""
    m = vfs.load_scene(str(GOLDEN / "scenes" / "dam_break.json"))
    counts = json.loads((GOLDEN / "scenes" / "expected_counts.json").read_text())
    assert m.n_particles == counts["dam_break.json"]
    sim, sph, wc = m.get_parameters()
    assert sph.iterations == 3 and abs(sim.smooth_radius - 0.2) < 1e-7
    s0 = m.copy_data_buffers()
    diam = np.cbrt(np.float32(1) / np.float32(1000.0)).astype(np.float32)
    assert np.allclose(s0["positions"][1] - s0["positions"][0], (0, 0, diam), atol=1e-6)
    assert np.allclose(s0["positions"][0], (0.0, 0.0, 1.5))
    from oracle import binding as ob

    o = ob.OracleModel(ob.params_from(sim, sph, wc), m.n_particles)
    o.set_state(s0["positions"], s0["velocities"])
    m.record_fields(True)
    m.step()
    o.step()
    assert np.array_equal(m.get_neighbor_arrays()[0], o.neighbors()[0])
    g, r = m.copy_data_buffers(), o.state()
    for k in ("positions", "velocities", "densities"):
        assert normwise_rel(g[k], r[k]) <= RTOL, k
    m.reset()
    assert np.array_equal(m.copy_data_buffers()["positions"], s0["positions"])


def test_partial_state_update_and_profile():
    w = W.dam_break(dims=(12, 12, 12), map_res=16)
    m = W.build_model(w)
    newp = w.pos[:100] + np.float32(0.01)
    m.set_particle_state(newp, np.ones((100, 3), np.float32), offset=500, count=100)
    s = m.copy_data_buffers()
    assert np.array_equal(s["positions"][500:600], newp)
    assert np.array_equal(s["positions"][:500], w.pos[:500])
    assert np.all(s["densities"][500:600] == 0)
    assert np.array_equal(m.get_ids()[500:600], np.arange(500, 600))
    prof = m.profile_substeps(3)
    assert all(v > 0 for k, v in prof.items() if k != "clear"), prof
    m.synchronize()
    with pytest.raises(vfs.VfsError):
        m.set_particle_state(newp, newp, offset=w.n - 10, count=100)


# 24,000 particles run the density pass three lanes per particle, 64,000 one lane.
@pytest.mark.parametrize("n_uniform", [20000, 60000])
def test_dense_cluster_overflows_the_neighbour_list(n_uniform):
    """A tight Gaussian cluster gives hundreds of neighbours per particle, more than the
    neighbour-list capacity: the force pass must fall back to its own candidate walk."""
    w = W.stress_4m(n_uniform=n_uniform, n_blob=4000, map_res=0)
    blob = vfs.generate_uniform_blob(0, (0, 0, 0), (1, 1, 1), 4000, (2.0, 1.0, 1.0), 0.008, 77)
    w.pos[n_uniform:] = blob
    m = W.build_model(w)
    o = oracle_for(w, m)
    compare_step(m, o, "dense_cluster")
    g = m.copy_data_buffers()
    assert g["densities"].max() > 50 * np.median(g["densities"])


@pytest.mark.parametrize("n_uniform", [20000, 60000])
def test_neighbour_capacity_changes_no_result(n_uniform):
    """The same dense cluster with 2048 list slots (no list overflows, so the force pass uses the
    lists) and with 128 (most blob particles fall back to the walk): bit-identical steps."""
    w = W.stress_4m(n_uniform=n_uniform, n_blob=4000, map_res=0)
    blob = vfs.generate_uniform_blob(0, (0, 0, 0), (1, 1, 1), 4000, (2.0, 1.0, 1.0), 0.008, 77)
    w.pos[n_uniform:] = blob
    a = W.build_model(w)
    b = W.build_model(w)
    assert a.neighbor_capacity == 128
    b.set_neighbor_capacity(2048)
    assert b.neighbor_capacity == 2048
    for m in (a, b):
        m.substeps(2)
    sa, sb = a.copy_data_buffers(), b.copy_data_buffers()
    for k in ("positions", "velocities", "densities"):
        assert np.array_equal(sa[k], sb[k]), k
    with pytest.raises(vfs.VfsError):
        b.set_neighbor_capacity(8)


def test_negative_cells_and_hash_block_boundaries():
    """Particles spanning cells -31..31 cross the uint wrap of cell + 25 (cells -26/-25) and the
    50-cell hash-block boundaries, where the candidate walk must not skip any bucket."""
    w = W.stress_4m(n_uniform=30000, n_blob=0, map_res=0)
    rng = np.random.default_rng(5)
    w.pos = ((rng.random((30000, 3)) - 0.5) * 1.25).astype(np.float32)
    w.sph = replace(w.sph, bbox_size=(2.0, 2.0, 2.0), bbox_pos=(-1.0, -1.0, -1.0))
    w.vel = ((rng.random((30000, 3)) - 0.5) * 0.2).astype(np.float32)
    m = W.build_model(w)
    o = oracle_for(w, m)
    for _ in range(2):
        compare_step(m, o, "negative_cells")


def test_incremental_sort_when_no_particle_changes_cell():
    """Zero gravity and velocity, particles held at rest in a lattice far from walls: after the
    first substep no key changes, the moved set is empty and the order must stay the stable sort."""
    w = W.dam_break(dims=(20, 20, 20), spacing=0.02, map_res=0, seed=3)
    w.sim = replace(w.sim, gravity=(0.0, 0.0, 0.0))
    w.pos = (w.pos + np.float32(0.1)).astype(np.float32)
    w.wcsph = replace(w.wcsph, stiffness=0.0, viscosity_strenght=0.0)
    m = W.build_model(w)
    o = oracle_for(w, m)
    for k in range(3):
        compare_step(m, o, f"no_moves_{k}", check_fields=False)


def test_incremental_sort_when_every_particle_changes_cell():
    """Velocities of about two cells per substep in random directions: nearly every key changes
    each substep, so the moved set is almost everything (and the merge has little to merge)."""
    w = W.dam_break(dims=(24, 24, 24), spacing=0.02, map_res=0, seed=8)
    w.sph = replace(w.sph, bbox_size=(4.0, 4.0, 4.0), bbox_pos=(-2.0, -2.0, -2.0))
    h, dt = float(w.sim.smooth_radius), float(w.sph.fixed_dt)
    rng = np.random.default_rng(9)
    w.vel = (rng.standard_normal(w.pos.shape) * (2.0 * h / dt)).astype(np.float32)
    w.wcsph = replace(w.wcsph, stiffness=0.0, viscosity_strenght=0.0)
    m = W.build_model(w)
    o = oracle_for(w, m)
    for k in range(3):
        compare_step(m, o, f"all_move_{k}", check_fields=False)
