"""CPU tests of the C ABI library: it loads, exports every declared entry point, and its host-only
logic (input generators, scene-JSON validation) behaves; no call here touches a GPU."""
from __future__ import annotations

import ctypes as C
import json
import re
from pathlib import Path

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from vkfluidsim_gb300 import _abi

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"


def declared_symbols():
    text = (ROOT / "include" / "vfs_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vfs_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(_abi.LIB_PATH))
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # ...and the Python binding declares a signature for each of them.
    assert sorted(_abi.SIGNATURES) == names


def test_version_and_last_error_are_callable_without_a_device():
    lib = vfs.load_library()
    assert b"sm_103a" in lib.vfs_version()
    assert lib.vfs_device_count() >= 0


def test_lattice_generator_is_deterministic_and_bounded():
    a = vfs.generate_lattice((5, 4, 3), (1.0, 2.0, 3.0), 0.1, 0.1, 42)
    b = vfs.generate_lattice((5, 4, 3), (1.0, 2.0, 3.0), 0.1, 0.1, 42)
    c = vfs.generate_lattice((5, 4, 3), (1.0, 2.0, 3.0), 0.1, 0.1, 43)
    assert a.shape == (60, 3) and np.array_equal(a, b) and not np.array_equal(a, c)
    ideal = vfs.generate_lattice((5, 4, 3), (1.0, 2.0, 3.0), 0.1, 0.0, 42)
    assert np.abs(a - ideal).max() <= 0.1 * 0.1 + 1e-6
    assert np.allclose(ideal[1] - ideal[0], (0.1, 0.0, 0.0), atol=1e-6)  # x fastest
    assert np.allclose(ideal[5] - ideal[0], (0.0, 0.1, 0.0), atol=1e-6)


def test_uniform_blob_generator():
    p = vfs.generate_uniform_blob(20000, (0, 0, 0), (4, 2, 2), 20000, (2, 1, 1), 0.1, 5)
    u, g = p[:20000], p[20000:]
    assert u.min() >= 0 and (u.max(0) <= (4, 2, 2)).all()
    assert np.allclose(g.mean(0), (2, 1, 1), atol=0.01)
    assert np.allclose(g.std(0), 0.1, rtol=0.05)


def test_fourier_velocity_generator():
    p = vfs.generate_lattice((16, 16, 16), (0, 0, 0), 0.02, 0.1, 1)
    v = vfs.generate_fourier_velocity(p, 8, 0.5, 9)
    sp = np.linalg.norm(v, axis=1)
    assert abs(sp.max() - 0.5) < 1e-5
    # Smooth: neighbouring lattice points have close velocities.
    assert np.abs(v[1] - v[0]).max() < 0.2


def _scene_error(tmp_path, text):
    p = tmp_path / "scene.json"
    p.write_text(text)
    with pytest.raises(vfs.VfsError) as e:
        vfs.load_scene(str(p))
    return e.value


def test_scene_json_errors_are_reported_not_thrown(tmp_path):
    assert _scene_error(tmp_path, "{ not json").code == 5
    err = _scene_error(tmp_path, json.dumps({"simulationParameters": {}}))
    assert err.code == 5 and "timeScale" in str(err)
    with pytest.raises(vfs.VfsError) as e:
        vfs.load_scene(str(tmp_path / "missing.json"))
    assert e.value.code == 4


def test_reference_scene_fixture_with_meshes_parses(tmp_path):
    """obstacle.json names two OBJ meshes: the JSON parses, and without a GPU the load stops at
    the model's creation (with one, tests/test_mesh.py loads it)."""
    err = _scene_error(tmp_path, (GOLDEN / "scenes" / "obstacle.json").read_text())
    assert err.code != 5, str(err)
