"""CPU-side descriptions of the benchmark workloads, for the oracle alone.

TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py's CPU legs (the reference arm among
them). It never imports the product package, so a process that times the oracle through it maps
no GPU library. The seeded lattice is a NumPy restatement of the product's counter-based
generator (splitmix64, ``vfs_generate_lattice``); a CPU test checks the two bit for bit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import binding as ob

SHAPE_SPHERE, SHAPE_BOX, SHAPE_CONTAINER = 0, 1, 2

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def u01(seed: int, index: np.ndarray) -> np.ndarray:
    """Uniform doubles in [0, 1): the top 53 bits of mix(mix(seed) ^ mix(index ^ c))."""
    s = _splitmix64(np.array([seed], np.uint64))[0]
    i = np.asarray(index, np.uint64) ^ np.uint64(0xD1B54A32D192ED03)
    r = _splitmix64(s ^ _splitmix64(i))
    return (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def lattice(dims, origin, spacing: float, jitter: float, seed: int) -> np.ndarray:
    """Jittered cubic lattice, x fastest: x = origin + spacing (idx + 0.5 + (2u - 1) jitter),
    evaluated in double and rounded to float once, as the product's generator does."""
    nx, ny, nz = (int(d) for d in dims)
    total = nx * ny * nz
    lin = np.arange(total, dtype=np.uint64)
    idx = np.stack([lin % np.uint64(nx), (lin // np.uint64(nx)) % np.uint64(ny),
                    lin // np.uint64(nx * ny)], axis=1).astype(np.float64)
    j = (2.0 * u01(seed, np.arange(3 * total, dtype=np.uint64)).reshape(total, 3) - 1.0) \
        * np.float64(np.float32(jitter))
    o = np.asarray(origin, np.float32).astype(np.float64)
    sp = np.float64(np.float32(spacing))
    return (o + sp * (idx + 0.5 + j)).astype(np.float32)


class Obstacle1M:
    """The 1,048,576-particle obstacle scene: a 128 x 128 x 64 lattice at spacing 0.0075 m
    (jitter 0.1 spacing, seed 1), h = 0.015 m, in a 2 x 1 x 1 m box with a sphere of radius 0.2 m
    at (1.4, 0.5, 0.2) given as a 128^3 volume map, rho0 = 1000, k = 50, gamma = 7, nu = 0.01,
    wall stiffness 1e4, g = -9.81 z, dt = 1e-4."""

    name = "obstacle_1m"
    dims = (128, 128, 64)
    spacing = 0.0075
    h = 0.015
    dt = 1e-4
    sphere_center = (1.4, 0.5, 0.2)
    sphere_radius = 0.2

    def __init__(self, seed: int = 1, map_res: int = 128):
        self.seed = seed
        self.map_res = map_res
        self.pos = lattice(self.dims, (0.0, 0.0, 0.0), self.spacing, 0.1, seed)
        self.vel = np.zeros_like(self.pos)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    def params(self) -> ob.OracleParams:
        return ob.OracleParams((C.c_float * 3)(0.0, 0.0, -9.81), self.h, 1.0, 1, self.dt, 1000.0,
                               (C.c_float * 3)(2.0, 1.0, 1.0), (C.c_float * 3)(0.0, 0.0, 0.0),
                               1e4, 50.0, 7.0, 0.01)

    def objects(self):
        """The sphere as a boundary object: grids from the oracle's volume-map generator (margin
        8 h, 16-point quadrature), built once."""
        if getattr(self, "_objects", None) is None:
            res = (self.map_res,) * 3
            bs, bp, sdf, vm = ob.volume_map(SHAPE_SPHERE, (self.sphere_radius,), self.h, res,
                                            np.float32(8.0 * self.h))
            t = np.eye(4, dtype=np.float32)
            t[:3, 3] = -np.asarray(self.sphere_center, np.float32)
            self._objects = [type("Obj", (), dict(
                transform=t.T.ravel(), rotation=np.eye(4, dtype=np.float32).ravel(), box_size=bs,
                box_pos=bp, resolution=res, sdf=sdf, volume_map=vm))]
        return self._objects

    def oracle(self) -> ob.OracleModel:
        """The oracle model of the scene at its initial state."""
        o = ob.OracleModel(self.params(), self.n)
        for info in self.objects():
            o.add_object(info)
        o.set_state(self.pos, self.vel)
        return o
