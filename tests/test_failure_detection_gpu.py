"""Failure detection without a GPU fault: the radix sort's look-back wait polls a predecessor's
status word a bounded number of times. In the self-test nothing ever publishes, so every waiting
thread gives up, sets the error word and returns; the host reads VFS_ERR_DEVICE_CHECK and the CUDA
context stays usable (a model steps correctly afterwards)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _selftest(published: int, spins: int):
    lib = vfs.load_library()
    err = C.c_uint32(0xFFFFFFFF)
    exc = (C.c_uint32 * 32)()
    rc = lib.vfs_selftest_lookback(published, spins, C.byref(err), exc)
    return rc, err.value, list(exc)


def test_wait_that_runs_out_reports_an_error_and_returns():
    rc, err, _ = _selftest(0, 1000)
    assert rc == 7  # VFS_ERR_DEVICE_CHECK
    assert err == 1  # look-back timeout bit
    assert b"look-back timeout" in vfs.load_library().vfs_last_error()


def test_published_predecessor_is_summed_without_error():
    rc, err, exc = _selftest(1, 1000)
    assert rc == 0 and err == 0
    assert exc == [b + 1 for b in range(32)]


def test_context_stays_usable_after_a_timeout():
    assert _selftest(0, 10)[0] == 7
    w = W.dam_break(dims=(12, 12, 12), map_res=0, seed=3)
    m = W.build_model(w)
    m.substeps(2)
    m.synchronize()  # raises if the model's own error word were set
    s = m.copy_data_buffers()
    assert np.isfinite(s["positions"]).all()


def test_spin_limit_is_validated():
    assert _selftest(0, 0)[0] == 1
    assert _selftest(0, (1 << 20) + 1)[0] == 1
