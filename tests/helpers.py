"""Comparison helpers and oracle construction shared by the tests.

Tolerances (FP32): a field matches when its normwise relative error
max_i |x_gpu - x_ref| / max_i |x_ref| is at most RTOL = 1e-5 (per field, all components). The
normwise form is used for accelerations and velocities because their per-element relative errors
are unbounded where a force nearly cancels (interior particles at rest) or where the Tait pressure
k((rho/rho0)^7 - 1) subtracts two nearly equal numbers. Densities (strictly positive, at least
m W(0)) and positions (coordinates of order the box) are also held element-wise:
|x_gpu - x_ref| <= RTOL * max(|x_ref|, floor) for every element, with floor = 0 for densities and
floor = h for position components (a coordinate near 0 is compared at the scale of h). The
FP32-vs-FP64 error of the oracle itself is reported beside it.
"""
from __future__ import annotations

import numpy as np

from oracle import binding as ob

RTOL = 1e-5


def normwise_rel(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.abs(b).max() if b.size else 0.0
    if scale == 0.0:
        return float(np.abs(a - b).max()) if a.size else 0.0
    return float(np.abs(a - b).max() / scale)


def elementwise_rel(a, b, floor: float = 0.0) -> float:
    """max_i |a_i - b_i| / max(|b_i|, floor) (0 where both are 0)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if not b.size:
        return 0.0
    den = np.maximum(np.abs(b), floor)
    d = np.abs(a - b)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(d == 0.0, 0.0, d / den)
    return float(r.max())


def elementwise_quantile(a, b, q: float, floor: float = 0.0) -> float:
    """The q-quantile of |a_i - b_i| / max(|b_i|, floor)."""
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    if not b.size:
        return 0.0
    den = np.maximum(np.abs(b), floor)
    d = np.abs(a - b)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(d == 0.0, 0.0, d / den)
    return float(np.quantile(r, q))


def oracle_for(workload, model=None, fp64=False, pos=None, vel=None, ids=None):
    """Oracle model of a workload with the GPU model's boundary grids (when given)."""
    o = ob.OracleModel(ob.params_from(workload.sim, workload.sph, workload.wcsph), workload.n,
                       fp64=fp64)
    if model is not None:
        for i in range(model.n_boundary_objects):
            o.add_object(model.get_boundary_object(i))
    o.set_state(workload.pos if pos is None else pos, workload.vel if vel is None else vel, ids)
    return o


def by_id(arr, ids):
    """Reorders a per-particle array from sorted order into id order."""
    out = np.empty_like(arr)
    out[ids] = arr
    return out
