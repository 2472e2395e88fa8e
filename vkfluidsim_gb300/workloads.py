"""Seeded synthetic scenes with the shapes of the benchmark configurations.

Each workload is a parameter set, a list of analytic boundary objects and an initial state; the
same description builds the GPU model and (in tests) the CPU oracle.

* ``dam_break_32k``  — 32^3 jittered lattice (spacing 0.02, jitter +-0.1 spacing) in the corner of
  a 1 m box, h = 0.04, rho0 = 1000, k = 50, gamma = 7, nu = 0.01, g = -9.81 z, dt = 2e-4, box walls
  as a 64^3 container volume map.
* ``obstacle_1m``    — 1,048,576 particles: a 128 x 128 x 64 lattice at spacing 0.0075 (h = 0.015)
  in a 2 x 1 x 1 m box holding a sphere of radius 0.2 (128^3 volume map), dt = 1e-4. (128^3
  particles at spacing 0.01 cannot give 1,048,576 particles nor fit the box, so the particle
  count is kept and the lattice is resized.)
* ``stress_4m``      — 4,194,304 uniform particles in 4 x 2 x 2 m plus 419,430 in a Gaussian blob
  (sigma = 0.1 m), h = 0.02, container volume map 128^3.
* ``dam_break_64k``  — 65,536 particles (64 x 32 x 32 lattice, spacing 0.0275, h = 0.06, 70% of the
  particles above rest density) in a 3 x 1.5 x 1.5 m box, dt = 2e-4, walls by the reference's
  penalty force only: the differentiable-rollout scene. Two choices keep its 300 substeps stable:
  the shader's gradient carries an extra 1/h, so the viscous term acts like a viscosity of about
  nu / h and explicit steps of 2e-4 blow up for h <= 0.04 at nu = 0.02; and a container volume map
  puts the boundary density near 1 at the walls (wall particles start near twice the rest density),
  which also blows up (the reference uses volume maps for obstacles only).
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import List

import numpy as np

from ._abi import SHAPE_CONTAINER, SHAPE_SPHERE
from .model import (AnalyticObject, SimulationParameters, SPHParameters, WCSPHParameters,
                    WCSPHWithBoundaryModel, generate_lattice, generate_uniform_blob)


@dataclass
class Workload:
    name: str
    sim: SimulationParameters
    sph: SPHParameters
    wcsph: WCSPHParameters
    objects: List[AnalyticObject]
    pos: np.ndarray
    vel: np.ndarray
    steps: int = 1
    notes: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


def _container(lo, hi, res) -> AnalyticObject:
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    c = 0.5 * (lo + hi)
    he = 0.5 * (hi - lo)
    return AnalyticObject(SHAPE_CONTAINER, tuple(he), position=tuple(float(x) for x in c),
                          resolution=tuple(res))


def dam_break(dims=(32, 32, 32), spacing=0.02, box=(1.0, 1.0, 1.0), map_res=64, dt=2e-4,
              stiffness=50.0, viscosity=0.01, seed=0, jitter=0.1, steps=200,
              name="dam_break") -> Workload:
    h = 2.0 * spacing
    pos = generate_lattice(dims, (0.0, 0.0, 0.0), spacing, jitter, seed)
    n = pos.shape[0]
    sim = SimulationParameters((0.0, 0.0, -9.81), h)
    sph = SPHParameters(1.0, 1, n, dt, 1000.0, box, (0.0, 0.0, 0.0))
    wc = WCSPHParameters(1e4, stiffness, 7.0, viscosity)
    objs = [_container((0, 0, 0), box, (map_res,) * 3)] if map_res else []
    return Workload(name, sim, sph, wc, objs, pos, np.zeros_like(pos), steps)


def dam_break_32k(**kw) -> Workload:
    return dam_break(name="dam_break_32k", **kw)


def obstacle_1m(map_res=128, seed=1, steps=1000) -> Workload:
    spacing = 0.0075
    h = 2.0 * spacing
    pos = generate_lattice((128, 128, 64), (0.0, 0.0, 0.0), spacing, 0.1, seed)
    n = pos.shape[0]
    sim = SimulationParameters((0.0, 0.0, -9.81), h)
    sph = SPHParameters(1.0, 1, n, 1e-4, 1000.0, (2.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    wc = WCSPHParameters(1e4, 50.0, 7.0, 0.01)
    sphere = AnalyticObject(SHAPE_SPHERE, (0.2,), position=(1.4, 0.5, 0.2),
                            resolution=(map_res,) * 3)
    return Workload("obstacle_1m", sim, sph, wc, [sphere], pos, np.zeros_like(pos), steps)


def stress_4m(n_uniform=4_194_304, n_blob=419_430, map_res=128, seed=2, steps=100) -> Workload:
    box = (4.0, 2.0, 2.0)
    pos = generate_uniform_blob(n_uniform, (0, 0, 0), box, n_blob, (2.0, 1.0, 1.0), 0.1, seed)
    n = pos.shape[0]
    sim = SimulationParameters((0.0, 0.0, -9.81), 0.02)
    sph = SPHParameters(1.0, 1, n, 1e-4, 1000.0, box, (0.0, 0.0, 0.0))
    wc = WCSPHParameters(1e4, 50.0, 7.0, 0.01)
    objs = [_container((0, 0, 0), box, (map_res,) * 3)] if map_res else []
    return Workload("stress_4m", sim, sph, wc, objs, pos, np.zeros_like(pos), steps)


def dam_break_64k(seed=4, steps=300) -> Workload:
    w = dam_break(dims=(64, 32, 32), spacing=0.0275, box=(3.0, 1.5, 1.5), map_res=0, dt=2e-4,
                  stiffness=50.0, viscosity=0.01, seed=seed, steps=steps, name="dam_break_64k")
    w.sim = replace(w.sim, smooth_radius=0.06)
    return w


def build_model(w: Workload) -> WCSPHWithBoundaryModel:
    """Creates the GPU model of a workload: parameters, boundary objects, initial state."""
    m = WCSPHWithBoundaryModel(w.sim, replace(w.sph, n_particles=w.n), w.wcsph)
    for o in w.objects:
        m.add_analytic_object(o)
    m.set_particle_state(w.pos, w.vel)
    return m


WORKLOADS = {
    "dam_break_32k": dam_break_32k,
    "obstacle_1m": obstacle_1m,
    "stress_4m": stress_4m,
    "dam_break_64k": dam_break_64k,
}


def batched_scenes(n_scenes=256, n_min=2048, n_max=65536, map_res=64, seed=3, steps=500):
    """Independent dam-break scenes of uneven size: N_s log-uniform in [n_min, n_max] (jittered
    lattices, spacing 0.02, h = 0.04, the column in the low corner octant of its own box), nu_s
    log-uniform in [1e-3, 5e-2], stiffness uniform in [20, 100], each with its own container volume
    map at map_res^3, dt = 2e-4."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_scenes)).astype(np.int64)
    nus = np.exp(rng.uniform(np.log(1e-3), np.log(5e-2), n_scenes))
    ks = rng.uniform(20.0, 100.0, n_scenes)
    spacing = 0.02
    out = []
    for s in range(n_scenes):
        n = int(sizes[s])
        side = int(np.ceil(np.cbrt(n)))
        nz = int(np.ceil(n / (side * side)))
        pos = generate_lattice((side, side, nz), (0.0, 0.0, 0.0), spacing, 0.1, seed * 100003 + s)[:n]
        box = (2 * side * spacing, 2 * side * spacing, 2 * nz * spacing)
        sim = SimulationParameters((0.0, 0.0, -9.81), 2 * spacing)
        sph = SPHParameters(1.0, 1, n, 2e-4, 1000.0, box, (0.0, 0.0, 0.0))
        wc = WCSPHParameters(1e4, float(ks[s]), 7.0, float(nus[s]))
        objs = [_container((0, 0, 0), box, (map_res,) * 3)] if map_res else []
        out.append(Workload(f"batch_scene_{s}", sim, sph, wc, objs, np.ascontiguousarray(pos),
                            np.zeros_like(pos), steps))
    return out


def build_batch(scenes):
    """One vfs_batch holding every workload of `scenes` (parameters, objects, initial state)."""
    from .model import Batch

    b = Batch([(w.sim, replace(w.sph, n_particles=w.n), w.wcsph) for w in scenes])
    for s, w in enumerate(scenes):
        for o in w.objects:
            b.add_analytic_object(s, o)
        b.set_particle_state(s, w.pos, w.vel)
    return b
