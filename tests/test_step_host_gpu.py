"""vfs_model_step_host (upload, substeps and read-back with one wait; with page-locked outputs the
last substep's density and force passes write them) must give exactly what set_particle_state +
substeps + copy_data_buffers give (SetParticleState, Step, CopyDataBuffers:
src/models/model.cpp:139-170).
Each case runs the same scene both ways over several host round trips, each round's output fed
back as the next round's input, and compares every output bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from vkfluidsim_gb300 import VfsError
from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _pinned(shape):
    import torch

    return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()


def _round_trips(w, rounds, substeps, pinned, keep_state_round=None):
    ref, fused = W.build_model(w), W.build_model(w)
    n = w.n
    pos, vel = np.array(w.pos, np.float32), np.array(w.vel, np.float32)
    pos_f, vel_f = pos.copy(), vel.copy()
    out = None
    if pinned:
        out = {"positions": _pinned((n, 3)), "velocities": _pinned((n, 3)),
               "densities": _pinned((n,))}
    for r in range(rounds):
        keep = r == keep_state_round
        if not keep:
            ref.set_particle_state(pos, vel)
        ref.substeps(substeps)
        a = ref.copy_data_buffers()
        if keep:
            b = fused.step_host(None, None, substeps, out=out)
        else:
            b = fused.step_host(pos_f, vel_f, substeps, out=out)
        for k in ("positions", "velocities", "densities"):
            assert np.array_equal(a[k], b[k]), f"round {r}: {k}"
        assert np.array_equal(ref.get_ids(), fused.get_ids()), f"round {r}: ids"
        pos, vel = a["positions"].copy(), a["velocities"].copy()
        pos_f, vel_f = b["positions"].copy(), b["velocities"].copy()
    return ref, fused


@pytest.mark.parametrize("pinned", [True, False])
def test_step_host_equals_the_three_calls(pinned):
    w = W.dam_break(dims=(40, 40, 40), map_res=32, stiffness=200.0)
    ref, fused = _round_trips(w, rounds=6, substeps=2, pinned=pinned, keep_state_round=3)
    assert ref.skin_builds() == fused.skin_builds()


def test_step_host_on_the_1m_scene_with_its_lists():
    w = W.obstacle_1m()
    ref, fused = _round_trips(w, rounds=4, substeps=3, pinned=True)
    assert fused.skin_builds() > 0


def test_round_trips_of_the_models_own_state_keep_its_skin_lists():
    """A frame loop that uploads the model's own state every substep renumbers the ids to the
    slots each time (SetParticleState sets ids to offset + i), while the sort has moved particles
    between slots. A whole-scene upload moves each slot's build index to the slot's new id, so
    the skin lists stay in use and the loop steps exactly like plain substeps: a round trip that
    fell back to the bucket walk would sum in another order and differ in the last bits."""
    w = W.obstacle_1m()
    plain, looped = W.build_model(w), W.build_model(w)
    for m in (plain, looped):
        m.substeps(120)  # falling at ~0.12 m/s: particles cross cells every substep
    s = looped.copy_data_buffers()
    n = w.n
    bufs = {"positions": _pinned((n, 3)), "velocities": _pinned((n, 3)), "densities": _pinned((n,))}
    bufs["positions"][:] = s["positions"]
    bufs["velocities"][:] = s["velocities"]
    b0, b1 = plain.skin_builds(), looped.skin_builds()
    for _ in range(8):
        plain.substeps(1)
        looped.step_host(bufs["positions"], bufs["velocities"], 1, out=bufs)
    a = plain.copy_data_buffers()
    for k in ("positions", "velocities", "densities"):
        assert np.array_equal(a[k], bufs[k]), k
    assert plain.skin_builds() - b0 == looped.skin_builds() - b1


def test_step_host_on_a_small_model():
    # 32,768 particles: the three-lane density pass; the force pass is the same kernel.
    w = W.dam_break_32k()
    _round_trips(w, rounds=3, substeps=1, pinned=True)


def test_step_host_replays_one_substep_through_the_same_pinned_buffers():
    """The frame loop: page-locked buffers that are both input and output, one substep per call
    (captured once per set of buffers and replayed); a second set of buffers midway."""
    w = W.dam_break(dims=(48, 40, 40), map_res=32, stiffness=200.0)
    ref, fused = W.build_model(w), W.build_model(w)
    n = w.n
    bufs = []
    for _ in range(2):
        b = {"positions": _pinned((n, 3)), "velocities": _pinned((n, 3)), "densities": _pinned((n,))}
        bufs.append(b)
    bufs[0]["positions"][:] = w.pos
    bufs[0]["velocities"][:] = w.vel
    pos, vel = np.array(w.pos, np.float32), np.array(w.vel, np.float32)
    for r in range(8):
        if r == 4:  # switch to the second set of buffers, holding the same state
            for k in ("positions", "velocities"):
                bufs[1][k][:] = bufs[0][k]
        b = bufs[0 if r < 4 else 1]
        ref.set_particle_state(pos, vel)
        ref.substeps(1)
        a = ref.copy_data_buffers()
        fused.step_host(b["positions"], b["velocities"], 1, out=b)
        for k in ("positions", "velocities", "densities"):
            assert np.array_equal(a[k], b[k]), f"round {r}: {k}"
        pos, vel = a["positions"].copy(), a["velocities"].copy()


def test_replayed_round_trips_after_an_upload_of_part_of_the_scene():
    """An upload of part of the scene between replayed round trips (its ids may then repeat, so
    the next whole upload must not move build indices by id): the replayed graph is captured
    again, and every round still equals the three separate calls bit for bit."""
    w = W.dam_break(dims=(48, 40, 40), map_res=32, stiffness=200.0)
    ref, fused = W.build_model(w), W.build_model(w)
    n = w.n
    b = {"positions": _pinned((n, 3)), "velocities": _pinned((n, 3)), "densities": _pinned((n,))}
    b["positions"][:] = w.pos
    b["velocities"][:] = w.vel
    pos, vel = np.array(w.pos, np.float32), np.array(w.vel, np.float32)
    for r in range(8):
        if r == 4:  # the same values written back over part of the scene, in both models
            part = slice(1000, 3000)
            ref.set_particle_state(pos[part], vel[part], offset=1000, count=2000)
            fused.set_particle_state(b["positions"][part].copy(), b["velocities"][part].copy(),
                                     offset=1000, count=2000)
        ref.set_particle_state(pos, vel)
        ref.substeps(1)
        a = ref.copy_data_buffers()
        fused.step_host(b["positions"], b["velocities"], 1, out=b)
        for k in ("positions", "velocities", "densities"):
            assert np.array_equal(a[k], b[k]), f"round {r}: {k}"
        pos, vel = a["positions"].copy(), a["velocities"].copy()
    assert ref.skin_builds() == fused.skin_builds()


def test_step_host_rejects_bad_arguments():
    m = W.build_model(W.dam_break(dims=(8, 8, 8), map_res=0))
    with pytest.raises(VfsError):
        m.step_host(None, None, 0)
    with pytest.raises(ValueError):
        m.step_host(np.zeros((m.n_particles, 3), np.float32), None, 1)
    with pytest.raises(ValueError):
        m.step_host(np.zeros((3, 3), np.float32), np.zeros((3, 3), np.float32), 1)
    with pytest.raises(ValueError):
        m.step_host(None, None, 1, out={"densities": np.zeros(3, np.float64)})
