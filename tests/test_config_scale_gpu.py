"""GPU parity at the benchmark configurations' own sizes.

* The 1,048,576-particle obstacle scene over its whole configured run of 1000 substeps: at
  substeps 100, 200, ..., 1000 the state is copied, the oracle steps once from it, and the GPU's
  sorted keys, sorted indices and spatial offsets must be bit-exact, its fields within the
  parity bars (tests/helpers.py compare_step: 1e-5 normwise, densities and positions also
  element-wise). From substep ~250 the configured run is blown apart (every particle changes
  cell every substep, speeds of order 1e5 m/s); those checkpoints cover that state.
* The 32,768-particle dam break as configured (32^3 lattice at 0.02 m, h = 0.04, 64^3 box-wall
  volume map, dt = 2e-4, 200 substeps): the same per-substep check at substeps 50, 100, 150 and
  200, and the drift of the whole GPU run from the oracle's own 200-substep run.
* The 256-scene batch (scene sizes log-uniform in [2048, 65536], 64^3 map per scene): after the
  benchmark's warm-up substeps, one substep of every scene from the same state agrees with the
  same scene run alone as a plain model (neighbour arrays bit-exact, fields within the bars), the
  continuous runs drift by at most 1e-3, and a sample of scenes matches the oracle.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from tests.helpers import RTOL, by_id, compare_step, elementwise_rel, normwise_rel, oracle_for
from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _check_from_state(m, w, label):
    """One GPU substep against one oracle substep from the GPU's current state."""
    s = m.copy_data_buffers()
    o = oracle_for(w, m, pos=s["positions"], vel=s["velocities"], ids=m.get_ids())
    return compare_step(m, o, label), s


def test_obstacle_1m_every_100_substeps_of_the_configured_run():
    w = W.obstacle_1m()
    m = W.build_model(w)
    speeds = {}
    done = 0
    for k in range(1, 11):
        m.substeps(100 * k - 1 - done)  # the compared substep is substep 100 k
        errs, s = _check_from_state(m, w, f"obstacle_1m substep {100 * k}")
        done = 100 * k
        speeds[done] = float(np.linalg.norm(s["velocities"], axis=1).max())
    print("obstacle_1m peak speed by substep (m/s):", json.dumps(speeds))
    assert done == w.steps == 1000
    assert m.skin_builds() >= 1


def test_dam_break_32k_as_configured():
    w = W.dam_break_32k()
    assert (w.n, w.steps, w.objects[0].resolution) == (32768, 200, (64, 64, 64))
    m = W.build_model(w)
    o_run = oracle_for(w, m)
    done = 0
    for k in (50, 100, 150, 200):
        m.substeps(k - 1 - done)
        _check_from_state(m, w, f"dam_break_32k substep {k}")
        done = k
    o_run.substeps(200)
    g, r = m.copy_data_buffers(), o_run.state()
    drift = float(np.abs(by_id(g["positions"], m.get_ids()) - by_id(r["positions"], r["ids"])).max())
    travel = float(np.abs(by_id(g["positions"], m.get_ids()) - w.pos).max())
    print(f"dam_break_32k: drift from the oracle's own 200-substep run {drift:.3g} m "
          f"(max travel {travel:.3g} m)")
    assert travel > 1e-3
    assert drift < 1e-4


@pytest.fixture(scope="module")
def batch256():
    scenes = W.batched_scenes(n_scenes=256)
    b = W.build_batch(scenes)
    b.record_fields(True)
    b.substeps(5)  # the benchmark's warm-up substeps
    return {"scenes": scenes, "batch": b, "substeps": 5}


def test_batch_256_scenes_equal_each_scene_alone(batch256):
    """Per substep from an identical state: after the warm-up, every scene's state is loaded into
    a plain model of that scene, the batch and the plain models advance one substep, and each
    scene's neighbour arrays must be bit-exact and its fields within the bars (densities also
    element-wise). The continuous 5-substep runs of both are compared too (drift reported and
    bounded: the small plain models sum their densities over three lanes, the batch over one, so
    rounding differs and grows over substeps)."""
    scenes, b = batch256["scenes"], batch256["batch"]
    assert len(scenes) == 256 and sum(w.n for w in scenes) > 4_000_000
    assert batch256["substeps"] == 5
    states = [dict(b.copy_data_buffers(s), ids=b.get_ids(s)) for s in range(len(scenes))]
    b.substeps(1)
    batch256["substeps"] += 1
    worst, worst_ew, worst_drift = 0.0, 0.0, 0.0
    for s, w in enumerate(scenes):
        m = W.build_model(w)
        m.substeps(5)  # the continuous run, as a loop of plain models would do it
        c, cid, st = m.copy_data_buffers(), m.get_ids(), states[s]
        drift = max(normwise_rel(by_id(c[k], cid), by_id(st[k], st["ids"]))
                    for k in ("positions", "densities"))
        worst_drift = max(worst_drift, drift)
        assert drift <= 1e-3, (s, drift)
        m.set_particle_state(states[s]["positions"], states[s]["velocities"])
        m.record_fields(True)
        m.substeps(1)
        bk, bp, bo = b.get_neighbor_arrays(s)
        mk, mp, mo = m.get_neighbor_arrays()
        assert np.array_equal(bk, mk) and np.array_equal(bp, mp) and np.array_equal(bo, mo), s
        gb, gm = b.copy_data_buffers(s, with_acc=True), m.copy_data_buffers(with_acc=True)
        for k in gm:
            e = normwise_rel(gb[k], gm[k])
            worst = max(worst, e)
            assert e <= RTOL, (s, k, e)
        ew = elementwise_rel(gb["densities"], gm["densities"])
        worst_ew = max(worst_ew, ew)
        assert ew <= RTOL, (s, ew)
        del m
    print(f"256 scenes, one substep from the same state: worst normwise batch vs plain {worst:.3g}, "
          f"densities element-wise {worst_ew:.3g}; drift of the continuous 5-substep runs "
          f"{worst_drift:.3g}")


def test_batch_256_sample_against_the_oracle(batch256):
    scenes, b, done = batch256["scenes"], batch256["batch"], batch256["substeps"]
    sizes = np.array([w.n for w in scenes])
    sample = sorted({int(np.argmin(sizes)), int(np.argsort(sizes)[len(sizes) // 2]),
                     int(np.argmax(sizes))})
    for s in sample:
        w = scenes[s]
        m = W.build_model(w)  # the oracle takes the same boundary grids
        o = oracle_for(w, m)
        o.substeps(done)
        ok, op, oo = o.neighbors()
        bk, bp, bo = b.get_neighbor_arrays(s)
        assert np.array_equal(bk, ok) and np.array_equal(bp, op) and np.array_equal(bo, oo), s
        g, r = b.copy_data_buffers(s), o.state()
        errs = {k: normwise_rel(g[k], r[k]) for k in ("positions", "velocities", "densities")}
        print(f"scene {s} ({w.n} particles) vs oracle after {done} substeps:",
              json.dumps({k: float(f"{v:.3g}") for k, v in errs.items()}))
        for k, e in errs.items():
            assert e <= RTOL, (s, k, e)
