"""GPU test of vfs_sort_pairs_noalloc, the sort entry point that allocates nothing.

Callers such as a frame loop or a host framework that owns the GPU memory budget cannot let a
library call cudaMalloc (it can synchronise the device, fragment their pool or break a stream
capture); this entry point runs the same stable pair sort out of a fixed device array instead. The
test calls it through the C ABI and requires outputs identical to the allocating vfs_sort_pairs
(integer outputs: bit-exact) on two calls in a row with different sizes and key widths, so the
second call also shows that the shared array's leftovers from the first are cleared. It lives in
its own file, collected last, and passes alone in a fresh process as well as after the suite.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vkfluidsim_gb300 import load_library

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAX_PAIRS = 262144  # VFS_SORT_NOALLOC_MAX_PAIRS in include/vfs_cuda.h
CAPACITY_ERROR = 6  # VFS_ERR_CAPACITY


def _run(fn, keys: np.ndarray, max_value: int):
    n = keys.size
    d_keys = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    d_items = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    rc = fn(C.c_void_p(d_items.data_ptr()), C.c_void_p(d_keys.data_ptr()), n, max_value, None)
    torch.cuda.synchronize()
    return rc, d_items.cpu().numpy().view(np.uint32), d_keys.cpu().numpy().view(np.uint32)


def test_no_alloc_sort_matches_the_allocating_sort_twice_in_a_row():
    lib = load_library()
    cases = [(MAX_PAIRS, MAX_PAIRS - 1, 11), (70_001, 2**32 - 1, 12)]
    for n, max_value, seed in cases:
        keys = np.random.default_rng(seed).integers(0, max_value + 1, size=n,
                                                    dtype=np.uint64).astype(np.uint32)
        rc_ref, items_ref, keys_ref = _run(lib.vfs_sort_pairs, keys, max_value)
        rc_new, items_new, keys_new = _run(lib.vfs_sort_pairs_noalloc, keys, max_value)
        assert rc_ref == 0 and rc_new == 0, lib.vfs_last_error()
        err = C.c_uint32(7)
        assert lib.vfs_sort_pairs_status(None, C.byref(err)) == 0 and err.value == 0
        assert np.array_equal(items_new, items_ref)
        assert np.array_equal(keys_new, keys_ref)
        assert np.array_equal(items_new, np.argsort(keys, kind="stable").astype(np.uint32))


def test_no_alloc_sort_rejects_sizes_beyond_its_array():
    lib = load_library()
    d = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc = lib.vfs_sort_pairs_noalloc(C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()),
                                    MAX_PAIRS + 1, 7, None)
    assert rc == CAPACITY_ERROR
    assert b"at most" in lib.vfs_last_error()


def test_no_alloc_sort_leaves_device_memory_unchanged():
    # Free device memory is the same before and after many calls (after one warm-up call that
    # loads the module and looks up the array's address).
    lib = load_library()
    n = 50_000
    keys = np.random.default_rng(5).integers(0, n, size=n).astype(np.uint32)
    d_keys = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    d_items = torch.empty(n, dtype=torch.int32, device="cuda")
    args = (C.c_void_p(d_items.data_ptr()), C.c_void_p(d_keys.data_ptr()), n, n - 1, None)
    assert lib.vfs_sort_pairs_noalloc(*args) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(100):
        assert lib.vfs_sort_pairs_noalloc(*args) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
