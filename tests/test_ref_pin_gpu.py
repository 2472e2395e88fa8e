"""GPU parity against the reference itself: the CUDA path (through the C ABI) stepped from the
inputs of the reference-step fixtures (tests/golden/ref_step, outputs of the reference's own step
shaders compiled as C++), one WCSPHWithBoundaryModel::Step per comparison from the reference's own
state before that step.

Bars: sorted keys, sorted indices and spatial offsets bit-exact; every float field within 1e-5
normwise; densities within 1e-5 element-wise (tests/helpers.py). The element-wise maxima and
99.9th percentiles of every field are printed (position components relative to max(|x|, h)).
"""
from __future__ import annotations

import json

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from tests.helpers import RTOL, elementwise_quantile, elementwise_rel, normwise_rel
from tests.ref_fixtures import FLOAT_FIELDS, INT_FIELDS, Fixture, names

pytestmark = pytest.mark.gpu


def gpu_model(fx: Fixture, pos, vel):
    m = vfs.WCSPHWithBoundaryModel(*fx.product_params())
    for o in fx.objects:
        m.add_boundary_object(o["transform"], o["rotation"], o["box_size"], o["box_pos"],
                              o["resolution"], o["sdf"], o["volume_map"])
    m.set_particle_state(pos, vel)
    m.record_fields(True)
    return m


def gpu_snapshot(m):
    k, p, off = m.get_neighbor_arrays()
    g = m.copy_data_buffers(with_acc=True)
    bd, bg = m.get_boundary_fields()
    return {"keys": k, "sorted_indices": p, "offsets": off, "positions": g["positions"],
            "velocities": g["velocities"], "densities": g["densities"],
            "accelerations": g["accelerations"], "boundary_density": bd, "boundary_gradient": bg}


def compare(got, ref, h, label):
    for k in INT_FIELDS:
        assert np.array_equal(got[k], ref[k]), f"{label}: {k} differ from the reference"
    errs = {}
    for k in FLOAT_FIELDS:
        floor = h if k == "positions" else 0.0
        errs[k] = {"normwise": normwise_rel(got[k], ref[k]),
                   "elementwise_max": elementwise_rel(got[k], ref[k], floor),
                   "elementwise_p999": elementwise_quantile(got[k], ref[k], 0.999, floor)}
    print(label, json.dumps({k: {a: float(f"{b:.3g}") for a, b in v.items()} for k, v in errs.items()}))
    for k, e in errs.items():
        assert e["normwise"] <= RTOL, f"{label}: {k} normwise {e['normwise']:.3g}"
    assert errs["densities"]["elementwise_max"] <= RTOL, label
    return errs


@pytest.mark.parametrize("name", names())
def test_each_step_matches_the_reference_from_its_own_state(name):
    fx = Fixture(name)
    pos, vel = fx.pos0, fx.vel0
    for s, ref in enumerate(fx.snaps):
        m = gpu_model(fx, pos, vel)
        m.step()
        m.synchronize()
        compare(gpu_snapshot(m), ref, fx.h, f"{name} step {s + 1}")
        pos, vel = ref["positions"], ref["velocities"]


@pytest.mark.parametrize("name", ["box_dam_break", "three_iterations_wall"])
def test_continuous_run_stays_on_the_reference(name):
    """The GPU run continued from the fixture's initial state: neighbour arrays stay bit-exact with
    the reference's at every step; the fields drift (SPH trajectories amplify rounding), which is
    printed and bounded at 1e-5 normwise for positions and densities."""
    fx = Fixture(name)
    m = gpu_model(fx, fx.pos0, fx.vel0)
    for s, ref in enumerate(fx.snaps):
        m.step()
        m.synchronize()
        got = gpu_snapshot(m)
        for k in INT_FIELDS:
            assert np.array_equal(got[k], ref[k]), f"{name} continuous step {s + 1}: {k}"
        drift = {k: normwise_rel(got[k], ref[k]) for k in FLOAT_FIELDS}
        print(f"{name} continuous step {s + 1} drift:",
              json.dumps({k: float(f"{v:.3g}") for k, v in drift.items()}))
        assert drift["positions"] <= RTOL and drift["densities"] <= RTOL


@pytest.mark.parametrize("name", ["icosphere", "box", "l_prism", "bumpy_sphere"])
def test_gpu_mesh_volume_map_matches_the_reference(name):
    """The GPU's mesh SDF grid and volume map (vfs_model_add_mesh_object) against the reference's
    own MeshSDF + GenerateVolumeMap (tests/golden/ref_volume_map): same grid box, SDF within 1e-6
    (FP64 distances rounded to float), volume map within 1e-5 of its largest value (the GPU
    evaluates the quadrature's integrand in FP32 and sums it in FP64)."""
    from pathlib import Path

    from vkfluidsim_gb300 import workloads as W

    z = np.load(Path(__file__).resolve().parent / "golden" / "ref_volume_map" / f"{name}.npz")
    h = float(z["h"])
    w = W.dam_break(dims=(4, 4, 4), map_res=0)
    from dataclasses import replace

    w.sim = replace(w.sim, smooth_radius=h)
    m = W.build_model(w)
    m.add_mesh_object(vfs.MeshObject(vertices=z["vertices"], triangles=z["triangles"],
                                     resolution=tuple(int(r) for r in z["resolution"])))
    g = m.get_boundary_object(0)
    assert np.array_equal(g.box_size, z["box_size"]) and np.array_equal(g.box_pos, z["box_pos"])
    e_sdf = float(np.abs(g.sdf - z["sdf"]).max())
    e_vm = float(np.abs(g.volume_map - z["volume_map"]).max() / np.abs(z["volume_map"]).max())
    print(f"{name}: sdf max |diff| {e_sdf:.3g} m, volume map {e_vm:.3g} of its maximum")
    assert e_sdf < 1e-6 and e_vm <= 1e-5
