"""Writes the reference-step golden fixtures ``tests/golden/ref_step/*.npz``.

Usage: python tests/golden/make_ref_step_golden.py <path of the VkFluidSim source tree>

Each fixture is one seeded scene stepped by the reference's own WCSPH step code: its Slang compute
shaders compiled as C++ by ``oracle/ref_build.py`` and driven in the order of its host code
(``oracle/ref_binding.RefShaderModel``). A fixture holds the inputs (parameter block, initial
state, boundary objects with their grids) and, after each call of WCSPHWithBoundaryModel::Step,
the outputs: sorted keys, sorted indices, spatial offsets, positions, velocities, densities,
accelerations, boundary density and gradient. The boundary grids are inputs here (made by the
oracle's volume-map generator); the step itself is the reference's.

Only this script (through the recipe) reads the reference tree; tests read the fixtures.
"""
from __future__ import annotations

import ctypes as C
import platform
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

OUT = HERE / "ref_step"
FIELDS = ("keys", "sorted_indices", "offsets", "positions", "velocities", "densities",
          "accelerations", "boundary_density", "boundary_gradient")


def params_array(g, h, time_scale, iterations, fixed_dt, rho0, box_size, box_pos, wall_k,
                 stiffness, expoent, viscosity):
    return np.array([*g, h, time_scale, iterations, fixed_dt, rho0, *box_size, *box_pos, wall_k,
                     stiffness, expoent, viscosity], np.float64)


def params_struct(a):
    from oracle import binding as ob

    a = [float(x) for x in a]
    return ob.OracleParams((C.c_float * 3)(*a[0:3]), a[3], a[4], int(a[5]), a[6], a[7],
                           (C.c_float * 3)(*a[8:11]), (C.c_float * 3)(*a[11:14]), a[14], a[15],
                           a[16], a[17])


def rotation_matrix(angle_deg, axis):
    """Rotation about a unit axis (Rodrigues), as a 4x4 matrix."""
    ax = np.asarray(axis, np.float64)
    ax = ax / np.linalg.norm(ax)
    t = np.radians(angle_deg)
    k = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    r = np.eye(4)
    r[:3, :3] = np.eye(3) + np.sin(t) * k + (1 - np.cos(t)) * (k @ k)
    return r


def make_object(shape, prm, h, res, center, angle_deg=0.0, axis=(0, 0, 1), scale=(1, 1, 1)):
    """A boundary object as GenericScene packs it: transform = inverse(T R S), rotation = R, both
    column-major; grids from the oracle's analytic generator (object-local, margin 8 h)."""
    from oracle import binding as ob

    bs, bp, sdf, vm = ob.volume_map(shape, prm, h, (res,) * 3, np.float32(8.0 * h))
    t = np.eye(4)
    t[:3, 3] = center
    r = rotation_matrix(angle_deg, axis)
    s = np.diag([*scale, 1.0])
    inv = np.linalg.inv(t @ r @ s)
    return {"transform": inv.T.astype(np.float32).ravel(), "rotation": r.T.astype(np.float32).ravel(),
            "box_size": bs, "box_pos": bp, "resolution": np.array([res] * 3, np.uint32),
            "sdf": sdf, "volume_map": vm}


def cases():
    from oracle.workloads import lattice

    out = {}
    # A: the dam-break column of the reference's scenes in a box-wall volume map.
    h = 0.04
    pos = lattice((12, 12, 12), (0, 0, 0), 0.02, 0.1, 0)
    out["box_dam_break"] = dict(
        params=params_array((0, 0, -9.81), h, 1.0, 1, 2e-4, 1000.0, (0.6, 0.6, 0.6), (0, 0, 0),
                            1e4, 50.0, 7.0, 0.01),
        pos=pos, vel=np.zeros_like(pos), steps=4,
        objects=[make_object(2, (0.3, 0.3, 0.3), h, 24, (0.3, 0.3, 0.3))])
    # B: 5,600 particles (more than 5,102, where the GPU prunes neighbour cells) in a unit box
    # with a rotated sphere and a rotated, scaled box, random velocities.
    rng = np.random.default_rng(11)
    pos = (rng.random((5600, 3)) * (0.6, 0.6, 0.4) + (0.1, 0.1, 0.0)).astype(np.float32)
    vel = ((rng.random((5600, 3)) - 0.5) * 0.5).astype(np.float32)
    out["rotated_objects"] = dict(
        params=params_array((0, 0, -9.81), h, 1.0, 1, 2e-4, 1000.0, (1.0, 1.0, 1.0), (0, 0, 0),
                            1e4, 100.0, 7.0, 0.01),
        pos=pos, vel=vel, steps=2,
        objects=[make_object(2, (0.5, 0.5, 0.5), h, 24, (0.5, 0.5, 0.5)),
                 make_object(0, (0.12,), h, 24, (0.4, 0.4, 0.15), 30.0, (1, 1, 0)),
                 make_object(1, (0.1, 0.05, 0.08), h, 24, (0.2, 0.6, 0.1), -90.0, (0, 1, 0),
                             (1.0, 2.0, 1.0))])
    # C: negative cell coordinates and a small table (many keys shared by neighbouring cells).
    rng = np.random.default_rng(5)
    pos = (rng.random((600, 3)) * 0.25 - 0.2).astype(np.float32)
    vel = ((rng.random((600, 3)) - 0.5) * 0.2).astype(np.float32)
    out["negative_cells_small_table"] = dict(
        params=params_array((0, 0, -9.81), h, 1.0, 1, 2e-4, 1000.0, (0.6, 0.6, 0.6),
                            (-0.3, -0.3, -0.3), 1e4, 50.0, 7.0, 0.01),
        pos=pos, vel=vel, steps=2, objects=[])
    # D: three iterations per Step call (dt = time_scale * fixed_dt / iterations), particles
    # pressed against the floor so the wall penalty acts.
    pos = lattice((8, 8, 8), (0, 0, -0.01), 0.02, 0.1, 3)
    out["three_iterations_wall"] = dict(
        params=params_array((0, 0, -9.81), h, 2.0, 3, 3e-4, 1000.0, (0.4, 0.4, 0.4), (0, 0, 0),
                            1e4, 50.0, 7.0, 0.02),
        pos=pos, vel=np.zeros_like(pos), steps=2, objects=[])
    # E: a single particle.
    out["single_particle"] = dict(
        params=params_array((0, 0, -9.81), h, 1.0, 1, 2e-4, 1000.0, (1, 1, 1), (0, 0, 0), 1e4,
                            50.0, 7.0, 0.01),
        pos=np.array([[0.5, 0.5, 0.02]], np.float32), vel=np.zeros((1, 3), np.float32), steps=2,
        objects=[])
    return out


def run_case(c):
    from oracle.ref_binding import RefShaderModel

    n = c["pos"].shape[0]
    r = RefShaderModel(params_struct(c["params"]), n)
    for o in c["objects"]:
        r.add_object(type("Obj", (), o))
    r.set_state(c["pos"], c["vel"])
    snaps = []
    for _ in range(c["steps"]):
        r.step(1)
        snaps.append(r.state())
    return snaps


def save(name, c, snaps):
    d = {"params": c["params"], "pos0": c["pos"], "vel0": c["vel"],
         "n_objects": np.int32(len(c["objects"])), "steps": np.int32(c["steps"]),
         "host": np.array(platform.machine())}
    for i, o in enumerate(c["objects"]):
        for k, v in o.items():
            d[f"obj{i}_{k}"] = np.asarray(v)
    for s, snap in enumerate(snaps):
        for k in FIELDS:
            d[f"step{s + 1}_{k}"] = snap[k]
    np.savez_compressed(OUT / f"{name}.npz", **d)


def main(ref: Path):
    from oracle import ref_build

    ref_build.build(ref)
    OUT.mkdir(exist_ok=True)
    for name, c in cases().items():
        snaps = run_case(c)
        save(name, c, snaps)
        print(name, c["pos"].shape[0], "particles,", c["steps"], "steps")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ref_step_golden.py <path of the VkFluidSim "
                 "source tree>")
    main(Path(sys.argv[1]))
