"""CPU tests that pin the oracle to the reference itself.

The fixtures under tests/golden/ref_step/ hold outputs of the reference's own WCSPH step code: its
Slang compute shaders compiled as C++ (oracle/ref_build.py) and driven in the order of its host
code. The oracle, stepped from the same inputs, must reproduce them bit for bit on the host that
wrote them (x86_64; both are built without floating-point contraction), and within 1e-6
normwise elsewhere. Where the reference build itself is present (oracle/_ref, made from the
reference source tree), more seeded scenes are stepped through both side by side.
"""
from __future__ import annotations

import platform

import numpy as np
import pytest

from oracle import binding as ob
from tests.helpers import normwise_rel
from pathlib import Path

from tests.ref_fixtures import FLOAT_FIELDS, INT_FIELDS, Fixture, names


def oracle_snapshot(o):
    k, p, off = o.neighbors()
    s, f = o.state(), o.fields()
    return {"keys": k, "sorted_indices": p, "offsets": off, "positions": s["positions"],
            "velocities": s["velocities"], "densities": s["densities"],
            "accelerations": f["accelerations"], "boundary_density": f["boundary_density"],
            "boundary_gradient": f["boundary_gradient"]}


def check_equal(got, ref, exact, label):
    for k in INT_FIELDS:
        assert np.array_equal(got[k], ref[k]), f"{label}: {k} differ"
    for k in FLOAT_FIELDS:
        if exact:
            assert np.array_equal(got[k], ref[k]), \
                f"{label}: {k} not bit-equal (normwise {normwise_rel(got[k], ref[k]):.3g})"
        else:
            assert normwise_rel(got[k], ref[k]) <= 1e-6, f"{label}: {k}"


def test_fixture_set_is_complete():
    assert set(names()) >= {"box_dam_break", "rotated_objects", "negative_cells_small_table",
                            "three_iterations_wall", "single_particle"}


@pytest.mark.parametrize("name", names())
def test_oracle_reproduces_the_reference_step(name):
    fx = Fixture(name)
    o = ob.OracleModel(fx.oracle_params(), fx.n)
    for info in fx.object_infos():
        o.add_object(info)
    o.set_state(fx.pos0, fx.vel0)
    exact = platform.machine() == fx.host
    for s, ref in enumerate(fx.snaps):
        o.step()  # one WCSPHWithBoundaryModel::Step: `iterations` substeps
        check_equal(oracle_snapshot(o), ref, exact, f"{name} step {s + 1}")
    # The reference's outputs are themselves consistent: sorted keys, offsets of the first entry.
    ref = fx.snaps[-1]
    keys, offs = ref["keys"], ref["offsets"]
    assert np.all(keys[1:] >= keys[:-1])
    first = np.full(fx.n, fx.n, np.uint32)
    first[keys[::-1]] = np.arange(fx.n - 1, -1, -1, dtype=np.uint32)
    assert np.array_equal(offs, first)


def _ref_or_skip():
    from oracle import ref_binding as rb

    if not rb.available():
        pytest.skip("the reference build (oracle/_ref) is not present on this machine")
    return rb


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_the_reference_build_on_seeded_scenes(seed):
    rb = _ref_or_skip()
    import ctypes as C

    rng = np.random.default_rng(seed)
    n = int(rng.integers(200, 3000))
    h = float(rng.uniform(0.02, 0.06))
    lo = rng.uniform(-0.3, 0.1, 3)
    pos = (lo + rng.random((n, 3)) * rng.uniform(0.1, 0.4, 3)).astype(np.float32)
    vel = ((rng.random((n, 3)) - 0.5) * rng.uniform(0.0, 1.0)).astype(np.float32)
    prm = ob.OracleParams((C.c_float * 3)(0.0, 0.0, -9.81), h, 1.0, int(rng.integers(1, 4)),
                          float(rng.uniform(1e-4, 4e-4)), 1000.0, (C.c_float * 3)(1.0, 1.0, 1.0),
                          (C.c_float * 3)(*lo.astype(np.float32)), 1e4,
                          float(rng.uniform(20, 200)), 7.0, float(rng.uniform(1e-3, 5e-2)))
    o = ob.OracleModel(prm, n)
    r = rb.RefShaderModel(prm, n)
    bs, bp, sdf, vm = ob.volume_map(0, (0.1,), h, (20, 20, 20), np.float32(8 * h))
    t = np.eye(4, dtype=np.float32)
    t[:3, 3] = -(lo + 0.2).astype(np.float32)
    info = type("Obj", (), dict(transform=t.T.ravel(), rotation=np.eye(4, dtype=np.float32).ravel(),
                                box_size=bs, box_pos=bp, resolution=(20, 20, 20), sdf=sdf,
                                volume_map=vm))
    o.add_object(info)
    r.add_object(info)
    o.set_state(pos, vel)
    r.set_state(pos, vel)
    for s in range(3):
        o.step()
        r.step(1)
        check_equal(oracle_snapshot(o), r.state(), True, f"seed {seed} step {s + 1}")


# ---- the volume-map generator (the step's boundary input), pinned to the reference's CPU code

VM_DIR = Path(__file__).resolve().parent / "golden" / "ref_volume_map"


def vm_fixtures():
    return sorted(p.stem for p in VM_DIR.glob("*.npz"))


def test_volume_map_fixture_set_is_complete():
    assert set(vm_fixtures()) >= {"icosphere", "box", "l_prism", "bumpy_sphere"}


@pytest.mark.parametrize("name", vm_fixtures())
def test_oracle_mesh_volume_map_reproduces_the_reference(name):
    """The oracle's mesh SDF and volume map (BVH-free brute force, Eberly point-triangle
    distance, angle-weighted pseudonormals, 16-point Gauss-Legendre) against the reference's own
    MeshSDF + GenerateVolumeMap: grid box and both grids bit for bit on this host."""
    z = np.load(VM_DIR / f"{name}.npz")
    h = float(z["h"])
    res = tuple(int(r) for r in z["resolution"])
    bs, bp, sdf, vm = ob.mesh_volume_map(z["vertices"], z["triangles"], h, res, np.float32(8.0 * h))
    assert np.array_equal(bs, z["box_size"]) and np.array_equal(bp, z["box_pos"])
    if platform.machine() == "x86_64":
        assert np.array_equal(sdf, z["sdf"]), normwise_rel(sdf, z["sdf"])
        assert np.array_equal(vm, z["volume_map"]), normwise_rel(vm, z["volume_map"])
    else:
        assert normwise_rel(sdf, z["sdf"]) <= 1e-6 and normwise_rel(vm, z["volume_map"]) <= 1e-6
    assert (z["volume_map"] > 0).sum() > 100


@pytest.mark.parametrize("seed", [11, 12])
def test_oracle_mesh_volume_map_matches_the_reference_build(seed):
    from oracle import ref_binding as rb

    if not rb.volume_map_available():
        pytest.skip("the reference volume-map build (oracle/_ref) is not present on this machine")
    from tests.golden.make_ref_volume_map_golden import icosphere

    rng = np.random.default_rng(seed)
    v, t = icosphere(float(rng.uniform(0.1, 0.3)), 1)
    v = (v * (1.0 + 0.2 * rng.random((len(v), 1))) + rng.uniform(-1, 1, 3)).astype(np.float32)
    h = float(rng.uniform(0.02, 0.06))
    res = tuple(int(x) for x in rng.integers(8, 20, 3))
    a = rb.mesh_volume_map(v, t, h, res)
    b = ob.mesh_volume_map(v, t, h, res, np.float32(8.0 * h))
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
