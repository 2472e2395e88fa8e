"""CPU tests of the benchmark's reference arm inputs: the oracle-side workload description builds
the same seeded initial state as the product's generator, and neither it nor bench.py's module
scope loads the product package (the reference arm times the oracle alone)."""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("dims,origin,spacing,jitter,seed", [
    ((7, 5, 3), (0.1, -0.2, 0.3), 0.02, 0.1, 0),
    ((16, 16, 16), (0.0, 0.0, 0.0), 0.0275, 0.3, 9),
    ((1, 1, 1), (1.0, 2.0, 3.0), 0.5, 0.0, 123456789),
])
def test_numpy_lattice_is_bit_equal_to_the_product_generator(dims, origin, spacing, jitter, seed):
    import vkfluidsim_gb300 as vfs
    from oracle.workloads import lattice

    a = lattice(dims, origin, spacing, jitter, seed)
    b = vfs.generate_lattice(dims, origin, spacing, jitter, seed)
    assert a.dtype == np.float32 and a.shape == b.shape
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_obstacle_1m_initial_state_matches_the_gpu_workload():
    from oracle.workloads import Obstacle1M
    from vkfluidsim_gb300 import workloads as W

    a, b = Obstacle1M(), W.obstacle_1m()
    assert a.n == b.n == 1_048_576
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.vel, b.vel)
    assert a.h == b.sim.smooth_radius and a.dt == b.sph.fixed_dt
    assert tuple(b.objects[0].position) == a.sphere_center


def test_reference_arm_imports_do_not_load_the_product():
    code = ("import sys; sys.path.insert(0, %r); import bench; import oracle.workloads; "
            "bad = [m for m in sys.modules if m.startswith('vkfluidsim_gb300')]; "
            "print(bad); sys.exit(1 if bad else 0)" % str(ROOT))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 0, r.stdout + r.stderr
