"""Candidate lists with a skin (Verlet lists) against the oracle.

The density pass sums each particle's list instead of walking its 27 buckets while no particle of
the scene has moved more than h skin / 2 since the last build. The in-range sets must be the
reference's in every substep (neighbour arrays bit-exact, fields within the parity bar), builds
must follow the displacements (including state written through the device pointers), and
batched scenes must keep their own build schedule."""
from __future__ import annotations

import numpy as np
import pytest

from tests.helpers import RTOL, normwise_rel, oracle_for
from tests.helpers import compare_step
from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def moving_scene(seed=0, speed=0.5):
    """64,000 particles (one lane per particle in the density pass, so the lists apply) 0.2 m
    away from the container's walls, with random velocities, so that at a skin of 0.02 h the lists
    go stale every few substeps."""
    w = W.dam_break(dims=(40, 40, 40), box=(1.2, 1.2, 1.2), map_res=24, seed=seed)
    w.pos = (w.pos + np.float32(0.2)).astype(np.float32)
    rng = np.random.default_rng(seed)
    w.vel = ((rng.random(w.pos.shape) - 0.5) * 2.0 * speed).astype(np.float32)
    return w


@pytest.mark.parametrize("skin", [0.02, 0.0])
def test_lists_track_the_oracle_across_builds(skin):
    w = moving_scene(seed=1)
    m = W.build_model(w)
    m.set_skin(skin)
    assert abs(m.skin - skin) < 1e-7
    o = oracle_for(w, m)
    for s in range(16):
        compare_step(m, o, f"skin{skin}_substep_{s}")
    builds = m.skin_builds()
    if skin:
        # The first substep builds; the others only after h skin / 2 of displacement.
        assert 2 <= builds < 16, builds
    else:
        assert builds == 0


def test_lists_off_and_on_agree():
    w = moving_scene(seed=2)
    a, b = W.build_model(w), W.build_model(w)
    a.set_skin(0.0)
    b.set_skin(0.02)
    assert a.skin == 0.0 and b.skin > 0.0
    a.substeps(12)
    b.substeps(12)
    assert a.skin_builds() == 0 and 1 <= b.skin_builds() < 12
    for x, y in zip(a.get_neighbor_arrays(), b.get_neighbor_arrays()):
        assert np.array_equal(x, y)
    sa, sb = a.copy_data_buffers(), b.copy_data_buffers()
    for k in ("positions", "velocities", "densities"):
        assert normwise_rel(sb[k], sa[k]) <= RTOL, k


class _DeviceRows:
    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n, 4), "typestr": "<f4", "data": (ptr, False),
                                         "version": 2}


def test_device_pointer_edits_keep_or_invalidate_the_lists():
    """A small edit keeps the lists (no new build, still the oracle's step); a large one makes the
    scene stale, so it walks (the oracle's step again)."""
    torch = pytest.importorskip("torch")
    w = moving_scene(seed=3, speed=0.05)
    m = W.build_model(w)
    m.set_skin(0.1)  # stale after 0.05 h of displacement
    m.substeps(2)
    assert m.skin_builds() == 1
    h = w.sim.smooth_radius
    g = torch.Generator(device="cuda").manual_seed(0)
    for shift in (0.02 * h, 0.5 * h):
        m.synchronize()
        p, _ = m.device_state()
        P = torch.as_tensor(_DeviceRows(p, w.n), device="cuda")
        P[:, :3] += (torch.rand((w.n, 3), device="cuda", generator=g) - 0.5) * (2.0 * shift / 3 ** 0.5)
        torch.cuda.synchronize()
        s = m.copy_data_buffers()
        o = oracle_for(w, m, pos=s["positions"], vel=s["velocities"], ids=m.get_ids())
        compare_step(m, o, f"device_edit_{shift / h:.2f}h")
        if shift < 0.05 * h:
            assert m.skin_builds() == 1


def test_batched_scenes_keep_their_own_builds():
    fast, slow = moving_scene(seed=4, speed=1.0), moving_scene(seed=5, speed=0.0)
    b = W.build_batch([fast, slow])
    b.set_skin(0.02)
    b.substeps(16)
    nf, ns = b.skin_builds(0), b.skin_builds(1)
    assert nf > ns >= 1, (nf, ns)
    # Each scene equals a plain model of it, which builds on the same schedule.
    for s, w in enumerate((fast, slow)):
        m = W.build_model(w)
        m.set_skin(0.02)
        m.substeps(16)
        assert m.skin_builds() == b.skin_builds(s)
        for x, y in zip(b.get_neighbor_arrays(s), m.get_neighbor_arrays()):
            assert np.array_equal(x, y)
        sb, sm = b.copy_data_buffers(s), m.copy_data_buffers()
        for k in ("positions", "velocities", "densities"):
            assert np.array_equal(sb[k], sm[k]), (s, k)


def test_fast_flow_backs_off_building():
    """Lists that go stale within a few substeps of their build make the scene wait longer and
    longer before building again: a fast flow mostly walks, and still matches the oracle."""
    w = moving_scene(seed=7, speed=3.0)  # stale one substep after every build
    m = W.build_model(w)
    m.set_skin(0.02)
    m.substeps(40)
    builds = m.skin_builds()
    assert 2 <= builds <= 4, builds  # 8, then 16 stale substeps walked before each build
    s = m.copy_data_buffers()
    o = oracle_for(w, m, pos=s["positions"], vel=s["velocities"], ids=m.get_ids())
    for k in range(3):
        compare_step(m, o, f"fast_flow_{k}")


def test_skin_argument_checks():
    import vkfluidsim_gb300 as vfs

    m = W.build_model(moving_scene(seed=6))
    for bad in (-0.1, 0.6, float("nan")):
        with pytest.raises(vfs.VfsError):
            m.set_skin(bad)
    # Small models run the three-lane density pass and have no lists.
    small = W.build_model(W.dam_break(dims=(10, 10, 10), map_res=0))
    assert small.skin == 0.0
    small.substeps(2)
    assert small.skin_builds() == 0


def test_single_scene_walkers_match_the_batched_walk():
    """A single scene's queued particles (no usable list) are walked one warp per particle; a
    batch walks them one thread per particle. Both must give the same sums and lists bit for bit:
    the 1M obstacle scene (about 1% of its particles walk once its lists are built, near the
    sphere and at hash-block boundaries) alone and batched with a small second scene."""
    w = W.obstacle_1m()
    tiny = W.dam_break(dims=(10, 10, 10), map_res=0)
    m = W.build_model(w)
    b = W.build_batch([w, tiny])
    m.substeps(4)
    b.substeps(4)
    assert m.skin_builds() == b.skin_builds(0) >= 1
    for x, y in zip(b.get_neighbor_arrays(0), m.get_neighbor_arrays()):
        assert np.array_equal(x, y)
    sb, sm = b.copy_data_buffers(0), m.copy_data_buffers()
    for k in ("positions", "velocities", "densities"):
        assert np.array_equal(sb[k], sm[k]), k
