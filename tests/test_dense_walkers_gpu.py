"""A single scene whose skin lists leave a crowd of walkers (a dense blob: hundreds of neighbours
within h, more candidates than a list holds) sums its usable lists in the list pass and walks
the rest a warp per walker. Its results must equal the bucket walk's bit for bit: the scene is
stepped from the same state repeatedly (as the stress workload is), so after the first substep
builds the lists, the list pass sums in the walk's order, and every walker is walked exactly as
the walk kernel walks it."""
from __future__ import annotations

import numpy as np
import pytest

from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_dense_walker_queue_matches_the_walk():
    w = W.stress_4m(n_uniform=1_000_000, n_blob=200_000, map_res=64)
    lists, walk = W.build_model(w), W.build_model(w)
    walk.set_skin(0.0)
    for m in (lists, walk):
        m.set_neighbor_capacity(640)  # the blob's in-range neighbours fit the force lists
    for r in range(3):
        for m in (lists, walk):
            m.set_particle_state(w.pos, w.vel)
            m.substeps(1)
        a, b = lists.copy_data_buffers(), walk.copy_data_buffers()
        for k in ("positions", "velocities", "densities"):
            assert np.array_equal(a[k], b[k]), f"repeat {r}: {k}"
        for x, y in zip(lists.get_neighbor_arrays(), walk.get_neighbor_arrays()):
            assert np.array_equal(x, y), f"repeat {r}: neighbour arrays"
    assert lists.skin_builds() == 1  # built once, then summed from the lists and the walkers
