"""CPU tests of the oracle: pinned against the reference's own data where it has any, otherwise
against independent restatements and the documented semantics of the reference shaders."""
from __future__ import annotations

import json
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

from oracle import binding as ob
from tests.helpers import normwise_rel
from vkfluidsim_gb300 import SHAPE_CONTAINER, SHAPE_SPHERE, workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden"
M32 = 0xFFFFFFFF


def py_hash(cx, cy, cz):
    """HashCell3D (spatial_hash_3d.slang:20-28) restated with Python integers mod 2^32."""
    u = [(c + 25) & M32 for c in (cx, cy, cz)]
    loc = [x % 50 for x in u]
    blk = [x // 50 for x in u]
    bh = (blk[0] * 15823 + blk[1] * 9737333 + blk[2] * 440817757) & M32
    return (loc[0] + 50 * (loc[1] + 50 * loc[2]) + bh) & M32


def py_keys(pos, h, n):
    cells = np.floor(pos.astype(np.float32) / np.float32(h)).astype(np.int64)
    return np.array([py_hash(*c) % n for c in cells], np.uint32)


def cubic_w(r, h):
    q = r / h
    s = 8.0 / (np.pi * h ** 3)
    return np.where(q <= 1, np.where(q > 0.5, 2 * s * (1 - q) ** 3, s * (6 * q ** 3 - 6 * q ** 2 + 1)), 0.0)


def cubic_dw(r, h):
    """Gradient magnitude with the shader's scale 48/(pi h^4)/h (kernels_3d.slang:78-91)."""
    q = r / h
    s = 48.0 / (np.pi * h ** 4) / h
    return np.where((r > 1e-9) & (q <= 1), np.where(q > 0.5, -s * (1 - q) ** 2, s * q * (3 * q - 2)), 0.0)


def test_gauss_legendre_matches_reference_table():
    g = json.loads((GOLDEN / "gauss_legendre_16.json").read_text())
    x, w = ob.gauss_legendre(16)
    ref = sorted(zip(g["abscissae"], g["weights"]))
    assert np.abs(np.sort(x) - np.array([a for a, _ in ref])).max() < 1e-14
    order = np.argsort(x)
    assert np.abs(w[order] - np.array([b for _, b in ref])).max() < 1e-14


def test_hash_matches_independent_restatement():
    rng = np.random.default_rng(0)
    cells = rng.integers(-300, 300, size=(2000, 3)).tolist()
    cells += [[-26, 0, 0], [-25, -25, -25], [2**31 - 1, 0, -2**31], [24, 24, 24], [25, 0, 0]]
    for c in cells:
        assert ob.hash_cell(*c) == py_hash(*c)


def test_hash_is_x_linear_inside_a_block():
    for cx in range(-25, 24):  # local x = cx + 25 in [0, 48]
        assert ob.hash_cell(cx + 1, 3, -7) == (ob.hash_cell(cx, 3, -7) + 1) & M32
    assert ob.hash_cell(25, 0, 0) != ob.hash_cell(24, 0, 0) + 1  # block boundary


def test_cell_coord_floor_and_saturation():
    assert ob.cell_coord(-0.01, 0.04) == -1
    assert ob.cell_coord(0.04, 0.04) == 1
    assert ob.cell_coord(0.0399999, 0.04) == 0
    assert ob.cell_coord(float("nan"), 0.04) == 0
    assert ob.cell_coord(1e30, 0.04) == 2**31 - 1
    assert ob.cell_coord(-1e30, 0.04) == -2**31


def _small_scene(n_side=12, map_res=0, **kw):
    return W.dam_break(dims=(n_side,) * 3, map_res=map_res, **kw)


def test_stable_sort_keys_and_offsets():
    w = _small_scene(14)
    rng = np.random.default_rng(3)
    pos = w.pos[rng.permutation(w.n)]  # scrambled input order
    o = ob.OracleModel(ob.params_from(w.sim, w.sph, w.wcsph), w.n)
    o.set_state(pos, w.vel)
    o.substeps(1)
    keys, perm, offs = o.neighbors()
    expected_keys = py_keys(pos, w.sim.smooth_radius, w.n)
    assert np.array_equal(np.sort(perm), np.arange(w.n))
    assert np.array_equal(keys, expected_keys[perm])
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    same = keys[1:] == keys[:-1]
    assert np.all(perm[1:][same] > perm[:-1][same]), "counting sort must be stable"
    first = np.full(w.n, w.n, np.uint32)
    for i in range(w.n - 1, -1, -1):
        first[keys[i]] = i
    assert np.array_equal(offs, first)


def test_duplicate_keys_are_walked_twice():
    """A tiny table (N = 29) makes neighbour cells collide; the density must count every particle
    of a duplicated key once per occurrence among the 27 keys (slang:166-190)."""
    n = 29
    rng = np.random.default_rng(7)
    h = 0.1
    pos = (rng.random((n, 3)) * 0.25).astype(np.float32)
    w = _small_scene(2)
    sim = replace(w.sim, smooth_radius=h)
    sph = replace(w.sph, n_particles=n)
    o = ob.OracleModel(ob.params_from(sim, sph, w.wcsph), n)
    o.set_state(pos, np.zeros_like(pos))
    o.substeps(1)
    s = o.state()
    # Brute force in float64 over the sorted input state with explicit multiplicities.
    keys, perm, _ = o.neighbors()
    x = pos[perm].astype(np.float64)
    mass = 1000.0 * 0.8 * h ** 3 / 8.0
    dens = np.zeros(n)
    dup_hits = 0
    for i in range(n):
        c = np.floor(np.float32(x[i]) / np.float32(h)).astype(np.int64)
        nk = [py_hash(c[0] + dx, c[1] + dy, c[2] + dz) % n
              for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
        for j in range(n):
            r = np.linalg.norm(x[j] - x[i])
            mult = nk.count(int(keys[j]))
            if r * r <= h * h and mult:
                dens[i] += mult * mass * float(cubic_w(r, h))
                dup_hits += mult > 1
    assert dup_hits > 0, "test scene must exercise a duplicated key"
    assert normwise_rel(s["densities"], dens) < 1e-5


def test_viscosity_uses_the_shader_gradient_scale():
    """Two particles, no gravity, no walls: the viscous acceleration follows
    10 nu (m / rho_j)(v_ij . x_ij) grad W / (r^2 + 0.01 h^2) with grad W scaled by 48/(pi h^5)."""
    h, nu = 0.1, 0.05
    w = _small_scene(2)
    sim = replace(w.sim, gravity=(0.0, 0.0, 0.0), smooth_radius=h)
    sph = replace(w.sph, n_particles=2, bbox_size=(10, 10, 10), bbox_pos=(-5, -5, -5))
    wc = replace(w.wcsph, viscosity_strenght=nu, stiffness=0.0)
    pos = np.array([[0.0, 0.0, 0.0], [0.06, 0.0, 0.0]], np.float32)
    vel = np.array([[0.0, 0.0, 0.0], [-1.0, 0.0, 0.0]], np.float32)
    o = ob.OracleModel(ob.params_from(sim, sph, wc), 2)
    o.set_state(pos, vel)
    o.substeps(1)
    s, f = o.state(), o.fields()
    ids = s["ids"]
    acc = np.empty((2, 3))
    acc[ids] = f["accelerations"]
    mass = 1000.0 * 0.8 * h ** 3 / 8.0
    rho = mass * (cubic_w(0.0, h) + cubic_w(0.06, h))
    xij = pos[0] - pos[1]
    r = np.linalg.norm(xij)
    vij = vel[0] - vel[1]
    expected = 10 * nu * (mass / rho) * np.dot(vij, xij) * (xij / r) * cubic_dw(r, h) / (r * r + 0.01 * h * h)
    assert normwise_rel(acc[0], expected) < 1e-5
    # The reference's CPU kernel (src/util/kernel.cpp:41-47) would give 1/h less: it is not used.
    assert normwise_rel(acc[0], expected * h) > 0.5


def _container_object(lo, hi, h, res):
    c = 0.5 * (np.asarray(lo) + np.asarray(hi))
    he = 0.5 * (np.asarray(hi) - np.asarray(lo))
    bs, bp, sdf, vm = ob.volume_map(SHAPE_CONTAINER, he, h, res, np.float32(8.0 * h))
    T = np.eye(4, dtype=np.float32)
    T[:3, 3] = -c  # world -> local translation
    return type("Obj", (), dict(transform=T.T.ravel(), rotation=np.eye(4, dtype=np.float32).ravel(),
                                box_size=bs, box_pos=bp, resolution=tuple(res), sdf=sdf,
                                volume_map=vm))


def test_fp32_restatement_tracks_the_fp64_twin():
    w = _small_scene(16, stiffness=200.0)
    pos = w.pos.copy()
    pos[:, 2] -= 0.004  # a few particles below the floor: wall penalty and boundary terms
    objs = [_container_object((0, 0, 0), (1, 1, 1), w.sim.smooth_radius, (24, 24, 24))]
    res = {}
    for fp64 in (False, True):
        o = ob.OracleModel(ob.params_from(w.sim, w.sph, w.wcsph), w.n, fp64=fp64)
        for ob_ in objs:
            o.add_object(ob_)
        o.set_state(pos, w.vel)
        o.substeps(3)
        s = o.state()
        res[fp64] = {k: s[k][np.argsort(s["ids"])] for k in ("positions", "velocities", "densities")}
        res[fp64]["bd"] = o.fields()["boundary_density"]
    assert res[False]["bd"].max() > 0, "scene must touch the volume map"
    assert normwise_rel(res[False]["densities"], res[True]["densities"]) < 1e-5
    assert normwise_rel(res[False]["velocities"], res[True]["velocities"]) < 1e-4
    assert normwise_rel(res[False]["positions"], res[True]["positions"]) < 1e-6


def test_volume_map_values():
    h = 0.02
    r0 = 0.1
    bs, bp, sdf, vm = ob.volume_map(SHAPE_SPHERE, [r0], h, (20, 20, 20), np.float32(8 * h))
    assert np.allclose(bs, 2 * r0 + 16 * h) and np.allclose(bp, -r0 - 8 * h)
    full_ball = 0.8 * 4.0 / 3.0 * np.pi * h ** 3
    deep = sdf < -1.5 * h
    assert deep.any()
    # 16^3 Gauss-Legendre points on the discontinuous ball indicator: a few per cent off the
    # exact ball volume, and the same value at every node deep inside the solid.
    assert np.abs(vm[deep] / full_ball - 1).max() < 0.05
    assert np.ptp(vm[deep]) == 0.0
    assert np.all(vm[sdf > 2 * h] == 0.0)
    near = (sdf > 0) & (sdf < 2 * h)
    assert np.all(vm[near] < full_ball) and np.all(vm[near] >= 0)
    # Monotone in the signed distance (spherical symmetry), up to the float rounding of the
    # node and quadrature points.
    order = np.argsort(sdf)
    assert np.all(np.diff(vm[order][sdf[order] < 2 * h]) <= 1e-4 * full_ball)


def test_grid_sampling_extrapolates_past_the_edge():
    """A particle within 0.1 h of the grid's edge: the central-difference probe leaves the grid;
    the oracle clamps the cell and extrapolates linearly (the reference reads out of bounds)."""
    h = 0.1
    res = (4, 4, 4)
    g = np.linspace(0.0, 1.0, 4)
    X, _, _ = np.meshgrid(g, g, g, indexing="ij")
    sdf = (0.3 * h + 0.5 * h * X).transpose(2, 1, 0).ravel().astype(np.float32)  # x fastest
    vm = np.ones(64, np.float32)
    obj = type("Obj", (), dict(transform=np.eye(4, dtype=np.float32).ravel(),
                               rotation=np.eye(4, dtype=np.float32).ravel(),
                               box_size=np.ones(3, np.float32), box_pos=np.zeros(3, np.float32),
                               resolution=res, sdf=sdf, volume_map=vm))
    w = _small_scene(2)
    sim = replace(w.sim, smooth_radius=h, gravity=(0, 0, 0))
    sph = replace(w.sph, n_particles=2, bbox_size=(10, 10, 10), bbox_pos=(-5, -5, -5))
    pos = np.array([[1.0 - 0.05 * h, 0.5, 0.5], [0.5, 0.5, 0.1]], np.float32)
    o = ob.OracleModel(ob.params_from(sim, sph, w.wcsph), 2)
    o.add_object(obj)
    o.set_state(pos, np.zeros_like(pos))
    o.substeps(1)
    s, f = o.state(), o.fields()
    i = int(np.where(s["ids"] == 0)[0][0])
    x = float(pos[0, 0])
    dist = 0.3 * h + 0.5 * h * x
    d = max(dist + 0.125 * h, 0.5 * h)
    assert abs(f["boundary_density"][i] - cubic_w(d, h)) / cubic_w(d, h) < 1e-5
    g_exp = np.array([cubic_dw(d, h), 0.0, 0.0])
    assert normwise_rel(f["boundary_gradient"][i], g_exp) < 1e-4
