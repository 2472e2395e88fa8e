"""Loader of the reference-step golden fixtures (tests/golden/ref_step/*.npz, written by
tests/golden/make_ref_step_golden.py from the reference's own step shaders compiled as C++)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

DIR = Path(__file__).resolve().parent / "golden" / "ref_step"
INT_FIELDS = ("keys", "sorted_indices", "offsets")
FLOAT_FIELDS = ("positions", "velocities", "densities", "accelerations", "boundary_density",
                "boundary_gradient")


def names():
    return sorted(p.stem for p in DIR.glob("*.npz"))


class Fixture:
    def __init__(self, name: str):
        z = np.load(DIR / f"{name}.npz")
        self.name = name
        self.params = z["params"]
        self.pos0 = z["pos0"]
        self.vel0 = z["vel0"]
        self.steps = int(z["steps"])
        self.host = str(z["host"])
        self.objects = []
        for i in range(int(z["n_objects"])):
            o = {k: z[f"obj{i}_{k}"] for k in ("transform", "rotation", "box_size", "box_pos",
                                                "resolution", "sdf", "volume_map")}
            o["resolution"] = tuple(int(x) for x in o["resolution"])
            self.objects.append(o)
        self.snaps = [{k: z[f"step{s}_{k}"] for k in INT_FIELDS + FLOAT_FIELDS}
                      for s in range(1, self.steps + 1)]

    @property
    def n(self) -> int:
        return int(self.pos0.shape[0])

    @property
    def h(self) -> float:
        return float(np.float32(self.params[3]))

    @property
    def iterations(self) -> int:
        return int(self.params[5])

    def oracle_params(self):
        from oracle import binding as ob

        a = [float(x) for x in self.params]
        return ob.OracleParams((C.c_float * 3)(*a[0:3]), a[3], a[4], int(a[5]), a[6], a[7],
                               (C.c_float * 3)(*a[8:11]), (C.c_float * 3)(*a[11:14]), a[14],
                               a[15], a[16], a[17])

    def object_infos(self):
        return [type("Obj", (), o) for o in self.objects]

    def product_params(self):
        """(SimulationParameters, SPHParameters, WCSPHParameters) of the product package."""
        import vkfluidsim_gb300 as vfs

        a = [float(x) for x in self.params]
        sim = vfs.SimulationParameters(tuple(a[0:3]), a[3])
        sph = vfs.SPHParameters(a[4], int(a[5]), self.n, a[6], a[7], tuple(a[8:11]),
                                tuple(a[11:14]))
        wc = vfs.WCSPHParameters(a[14], a[15], a[16], a[17])
        return sim, sph, wc
