"""The C++ adapter (include/vfs_gb300_model.hpp), compiled against include/vfs_cuda.h and linked
with the library as a maintainer would add it to the reference: a CPU test builds and runs it
(without a device the library's error surfaces as the adapter's exception), and a GPU test drives
one Step through it and compares the result with the oracle (neighbour arrays bit-exact, fields
within the parity bars) and with the same step taken by StepHost (bit for bit)."""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = Path(__file__).resolve().parent / "adapter" / "adapter_check.cpp"


def build(tmp_path: Path) -> Path:
    from vkfluidsim_gb300 import LIB_PATH

    exe = tmp_path / "adapter_check"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(SRC),
           f"-L{LIB_PATH.parent}", "-lvfs_cuda", f"-Wl,-rpath,{LIB_PATH.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_adapter_compiles_links_and_reports_errors(tmp_path):
    from vkfluidsim_gb300 import load_library

    exe = build(tmp_path)
    r = subprocess.run([str(exe), str(tmp_path / "out.bin")], capture_output=True, text=True,
                       timeout=120)
    if load_library().vfs_device_count() < 1:
        assert r.returncode == 3 and r.stdout.startswith("vfs: "), (r.returncode, r.stdout)
    else:
        assert r.returncode == 0, r.stdout


@pytest.mark.gpu
def test_adapter_step_matches_the_oracle(tmp_path):
    from oracle import binding as ob
    from tests.helpers import RTOL, normwise_rel

    exe = build(tmp_path)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    raw = out.read_bytes()
    n = int(np.frombuffer(raw[:4], np.uint32)[0])
    a = np.frombuffer(raw[4:], np.uint8)
    off = 0

    def take(dtype, count):
        nonlocal off
        v = np.frombuffer(a[off:off + count * np.dtype(dtype).itemsize].tobytes(), dtype)
        off += count * np.dtype(dtype).itemsize
        return v

    pos, vel = take(np.float32, 3 * n).reshape(n, 3), take(np.float32, 3 * n).reshape(n, 3)
    dens = take(np.float32, n)
    keys, perm, offs = take(np.uint32, n), take(np.uint32, n), take(np.uint32, n)
    # StepHost on a second model from the same lattice: the same results, bit for bit.
    pos2, vel2 = take(np.float32, 3 * n).reshape(n, 3), take(np.float32, 3 * n).reshape(n, 3)
    dens2 = take(np.float32, n)
    assert np.array_equal(pos2, pos) and np.array_equal(vel2, vel) and np.array_equal(dens2, dens)
    from oracle.workloads import lattice

    prm = ob.OracleParams((C.c_float * 3)(0.0, 0.0, -9.81), 0.04, 1.0, 1, 2e-4, 1000.0,
                          (C.c_float * 3)(0.4, 0.4, 0.4), (C.c_float * 3)(0.0, 0.0, 0.0), 1e4, 50.0,
                          7.0, 0.01)
    o = ob.OracleModel(prm, n)
    p0 = lattice((8, 8, 8), (0, 0, 0), 0.02, 0.1, 0)
    o.set_state(p0, np.zeros_like(p0))
    o.step()
    ok, op, oo = o.neighbors()
    assert np.array_equal(keys, ok) and np.array_equal(perm, op) and np.array_equal(offs, oo)
    s = o.state()
    for k, v in (("positions", pos), ("velocities", vel), ("densities", dens)):
        assert normwise_rel(v, s[k]) <= RTOL, k
