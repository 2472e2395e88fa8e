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

import json

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


def compare_step(model, oracle, label="", fp64_oracle=None, check_fields=True):
    """Runs one substep on both and checks the bars; returns the error table."""
    model.record_fields(True)
    model.substeps(1)
    oracle.substeps(1)
    gk, gp, go = model.get_neighbor_arrays()
    ok, op, oo = oracle.neighbors()
    assert np.array_equal(gk, ok), f"{label}: sorted keys differ"
    assert np.array_equal(gp, op), f"{label}: permutation differs"
    assert np.array_equal(go, oo), f"{label}: spatial offsets differ"
    g = model.copy_data_buffers(with_acc=True)
    o = oracle.state()
    assert np.array_equal(model.get_ids(), o["ids"])
    errs = {}
    if check_fields:
        bd, bg = model.get_boundary_fields()
        f = oracle.fields()
        errs["boundary_density"] = normwise_rel(bd, f["boundary_density"])
        errs["boundary_gradient"] = normwise_rel(bg, f["boundary_gradient"])
        errs["accelerations"] = normwise_rel(g["accelerations"], f["accelerations"])
    errs["densities"] = normwise_rel(g["densities"], o["densities"])
    errs["velocities"] = normwise_rel(g["velocities"], o["velocities"])
    errs["positions"] = normwise_rel(g["positions"], o["positions"])
    # Element-wise: densities relative to themselves (asserted); position components relative to
    # max(|x|, h) and velocity components relative to max(|v|, 1e-3 max|v|) (reported: a
    # particle's position and velocity errors follow its acceleration error, which is bounded
    # only normwise where forces nearly cancel or particles nearly coincide).
    h = float(model.get_parameters()[0].smooth_radius)
    vfloor = 1e-3 * max(float(np.abs(o["velocities"]).max()), 1e-30)
    ew = {"ew_densities": elementwise_rel(g["densities"], o["densities"]),
          "ew_p999_densities": elementwise_quantile(g["densities"], o["densities"], 0.999),
          "ew_positions": elementwise_rel(g["positions"], o["positions"], h),
          "ew_p999_positions": elementwise_quantile(g["positions"], o["positions"], 0.999, h),
          "ew_velocities": elementwise_rel(g["velocities"], o["velocities"], vfloor),
          "ew_p999_velocities": elementwise_quantile(g["velocities"], o["velocities"], 0.999,
                                                     vfloor)}
    if fp64_oracle is not None:
        fp64_oracle.substeps(1)
        d = fp64_oracle.state()
        for k in ("densities", "velocities", "positions"):
            ref = by_id(d[k], d["ids"])
            errs[f"gpu_vs_fp64_{k}"] = normwise_rel(by_id(g[k], o["ids"]), ref)
            errs[f"oracle32_vs_fp64_{k}"] = normwise_rel(by_id(o[k], o["ids"]), ref)
        ref = by_id(d["densities"], d["ids"])
        errs["gpu_vs_fp64_ew_densities"] = elementwise_rel(by_id(g["densities"], o["ids"]), ref)
        errs["oracle32_vs_fp64_ew_densities"] = elementwise_rel(by_id(o["densities"], o["ids"]), ref)
    print(label, json.dumps({k: float(f"{v:.3g}") for k, v in {**errs, **ew}.items()}))
    for k, v in errs.items():
        if not k.startswith(("gpu_vs_fp64", "oracle32_vs_fp64")):
            assert v <= RTOL, f"{label}: {k} normwise error {v:.3g} > {RTOL}"
    assert ew["ew_densities"] <= RTOL, f"{label}: densities element-wise {ew['ew_densities']:.3g}"
    errs.update(ew)
    return errs
