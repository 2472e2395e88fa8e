"""The differentiable-rollout test scene shared by the CPU and GPU adjoint tests.

5,832 particles (18^3 lattice at spacing 0.019, h = 0.04: slightly above rest density, so pressure
acts), a smooth initial velocity field (8 Fourier modes, 0.5 m/s), a 24^3 container volume map,
nu = 0.02, k = 20, dt = 1e-4, 12 substeps checkpointed every 5. N > 5102 and all cells inside one
50^3 hash block keep the 27 neighbour keys distinct, so no particle's neighbour multiplicity can
change under a small perturbation and the rollout is a smooth function of its inputs.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np

import vkfluidsim_gb300 as vfs
from vkfluidsim_gb300 import workloads as W

STEPS, EVERY = 12, 5


def scene():
    w = W.dam_break(dims=(18, 18, 18), spacing=0.019, map_res=24, stiffness=20.0,
                    viscosity=0.02, seed=7, dt=1e-4)
    w.sim = replace(w.sim, smooth_radius=0.04)
    w.vel = vfs.generate_fourier_velocity(w.pos, 8, 0.5, 11)
    return w


def target(w):
    return (w.pos + 0.01 * np.sin(7.0 * w.pos[:, [1, 2, 0]])).astype(np.float64)


def straddling_scene():
    """Scene A's lattice moved to x in [0.85, 1.19] inside a 2 x 1 x 1 container: cells 24..26 on
    x have neighbour cells in two 50^3 hash blocks, so particles with and without distinct neighbour
    keys interact (both the gathered and the scattered adjoint pair terms run)."""
    w = W.dam_break(dims=(18, 18, 18), spacing=0.019, box=(2.0, 1.0, 1.0), map_res=24,
                    stiffness=20.0, viscosity=0.02, seed=7, dt=1e-4)
    w.sim = replace(w.sim, smooth_radius=0.04)
    w.pos = (w.pos + np.array([0.85, 0.0, 0.0], np.float32)).astype(np.float32)
    w.vel = vfs.generate_fourier_velocity(w.pos, 8, 0.5, 11)
    return w


def small_scene():
    """1,440 particles (12 x 12 x 10): N <= 5102, so neighbour keys may collide everywhere and
    every adjoint pair term is scattered."""
    w = W.dam_break(dims=(12, 12, 10), spacing=0.019, map_res=24, stiffness=20.0,
                    viscosity=0.02, seed=5, dt=1e-4)
    w.sim = replace(w.sim, smooth_radius=0.04)
    w.vel = vfs.generate_fourier_velocity(w.pos, 8, 0.5, 13)
    return w


SCENES = {"one_block": scene, "straddling": straddling_scene, "small": small_scene}


def distinct_key_mask(w):
    """Per particle: are its 27 neighbour-cell keys certainly distinct (N > 5102 and all 27 cells
    in one 50^3 hash block, the condition the GPU kernels test)?"""
    c = np.floor(w.pos.astype(np.float64) / float(np.float32(w.sim.smooth_radius))).astype(np.int64)
    same = (((c + 24) // 50) == ((c + 26) // 50)).all(axis=1)
    return same & (w.n > 5102)


def cpu_objects(w):
    """The scene's boundary objects with grids from the oracle's CPU volume-map generator."""
    from oracle import binding as ob

    objs = []
    for a in w.objects:
        bs, bp, sdf, vm = ob.volume_map(a.shape, a.params, w.sim.smooth_radius, a.resolution,
                                        np.float32(8.0 * w.sim.smooth_radius))
        T = np.eye(4, dtype=np.float32)
        T[:3, 3] = -np.asarray(a.position, np.float32)
        objs.append(type("Obj", (), dict(
            transform=T.T.ravel(), rotation=np.eye(4, dtype=np.float32).ravel(), box_size=bs,
            box_pos=bp, resolution=tuple(a.resolution), sdf=sdf, volume_map=vm,
            n_boundary_objects=1)))
    return objs


class ObjectList:
    """Adapter giving a list of boundary objects the model's object-query interface."""

    def __init__(self, objs):
        self.objs = objs
        self.n_boundary_objects = len(objs)

    def get_boundary_object(self, k):
        return self.objs[k]


def torch_rollout(w, objects_source, nu, k, v0, steps=STEPS):
    """Final positions (by id) of the FP64 torch restatement; nu, k, v0 are torch tensors."""
    import torch

    from tests import fp64_torch_step as R

    P = R.params_of(w)
    objs = R.objects_of(objects_source)
    x = torch.from_numpy(w.pos.astype(np.float64))
    v = v0
    for _ in range(steps):
        x, v = R.substep(x, v, P, objs, nu, k)
    return x


def oracle_rollout(w, objects_source, nu, k, v0, steps=STEPS):
    """Final positions (by id) of the oracle's FP64 twin."""
    from oracle import binding as ob

    wc = replace(w.wcsph, viscosity_strenght=nu, stiffness=k)
    o = ob.OracleModel(ob.params_from(w.sim, w.sph, wc), w.n, fp64=True)
    for i in range(objects_source.n_boundary_objects):
        o.add_object(objects_source.get_boundary_object(i))
    o.set_state(w.pos.astype(np.float64), np.asarray(v0, np.float64))
    o.substeps(steps)
    s = o.state()
    xf = np.empty_like(s["positions"])
    xf[s["ids"]] = s["positions"]
    return xf
