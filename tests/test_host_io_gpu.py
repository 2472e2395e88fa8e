"""Host I/O through page-locked buffers: SetParticleState and CopyDataBuffers read and write
page-locked host memory directly from their conversion kernels, and pageable memory through a
staging copy. Both routes must give bit-identical states (model.cpp:137-160 semantics: a partial
range, the densities it covers zeroed, optional outputs)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vkfluidsim_gb300 import workloads as W
from vkfluidsim_gb300._abi import check

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def pinned(shape, dtype=torch.float32):
    return torch.zeros(shape, dtype=dtype, pin_memory=True)


def fptr(t):
    return None if t is None else C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_float))


def uptr(t):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_uint32))


def small_scene(seed=0):
    # 1,000 particles: not a multiple of the 256-record conversion block.
    return W.dam_break(dims=(10, 10, 10), spacing=0.02, box=(0.5, 0.5, 0.5), map_res=16, seed=seed)


def test_pinned_outputs_match_pageable():
    w = small_scene()
    m = W.build_model(w)
    m.substeps(3)
    ref = m.copy_data_buffers()
    ids_ref = m.get_ids()
    n = w.n
    hp, hv, hd = pinned((n, 3)), pinned((n, 3)), pinned((n,))
    check(m._lib.vfs_model_copy_data_buffers(m._h, fptr(hp), fptr(hv), fptr(hd), None))
    assert np.array_equal(hp.numpy(), ref["positions"])
    assert np.array_equal(hv.numpy(), ref["velocities"])
    assert np.array_equal(hd.numpy(), ref["densities"])
    hi = pinned((n,), torch.int32)
    check(m._lib.vfs_model_get_ids(m._h, uptr(hi)))
    assert np.array_equal(hi.numpy().view(np.uint32), ids_ref)
    # Optional outputs left out: only the positions are written.
    hp2 = pinned((n, 3))
    check(m._lib.vfs_model_copy_data_buffers(m._h, fptr(hp2), None, None, None))
    assert np.array_equal(hp2.numpy(), ref["positions"])


def test_pinned_inputs_match_pageable():
    w = small_scene(seed=1)
    a, b = W.build_model(w), W.build_model(w)
    a.substeps(2)
    b.substeps(2)
    rng = np.random.default_rng(7)
    off, cnt = 100, 557
    pos = (w.pos[off:off + cnt] + rng.normal(0, 1e-3, (cnt, 3))).astype(np.float32)
    vel = rng.normal(0, 0.1, (cnt, 3)).astype(np.float32)
    a.set_particle_state(pos, vel, offset=off, count=cnt)  # pageable: staging copy
    hp, hv = pinned((cnt, 3)), pinned((cnt, 3))
    hp.numpy()[:] = pos
    hv.numpy()[:] = vel
    check(b._lib.vfs_model_set_particle_state(b._h, fptr(hp), fptr(hv), off, cnt))
    sa, sb = a.copy_data_buffers(), b.copy_data_buffers()
    for k in ("positions", "velocities", "densities"):
        assert np.array_equal(sa[k], sb[k]), k
    a.substeps(2)
    b.substeps(2)
    sa, sb = a.copy_data_buffers(), b.copy_data_buffers()
    for k in ("positions", "velocities", "densities"):
        assert np.array_equal(sa[k], sb[k]), k


def test_pinned_batch_scene_io():
    scenes = [small_scene(seed=s) for s in range(3)]
    bt = W.build_batch(scenes)
    bt.substeps(2)
    s = 2  # a scene that does not start at particle 0
    ref = bt.copy_data_buffers(s)
    n = scenes[s].n
    hp, hv, hd = pinned((n, 3)), pinned((n, 3)), pinned((n,))
    check(bt._lib.vfs_batch_copy_data_buffers(bt._h, s, fptr(hp), fptr(hv), fptr(hd), None))
    assert np.array_equal(hp.numpy(), ref["positions"])
    assert np.array_equal(hv.numpy(), ref["velocities"])
    assert np.array_equal(hd.numpy(), ref["densities"])
    check(bt._lib.vfs_batch_set_particle_state(bt._h, s, fptr(hp), fptr(hv), 0, n))
    back = bt.copy_data_buffers(s)
    assert np.array_equal(back["positions"], ref["positions"])
    assert np.array_equal(back["velocities"], ref["velocities"])
    assert not back["densities"].any()  # SetParticleState zeroes the densities it covers


class _DeviceRows:
    """A (n, 4) float32 view of a device pointer for torch.as_tensor (no copy)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n, 4), "typestr": "<f4", "data": (ptr, False),
                                         "version": 2}


def test_state_edited_through_device_pointers_is_stepped():
    """Positions and velocities written in place through vfs_model_device_state are what the next
    substep steps: keys, permutation and offsets bit-exact and the fields within the parity bar
    against the oracle started from the edited state."""
    from tests.helpers import oracle_for
    from tests.helpers import compare_step

    w = small_scene(seed=3)
    m = W.build_model(w)
    m.substeps(2)
    m.synchronize()
    p, v = m.device_state()
    P = torch.as_tensor(_DeviceRows(p, w.n), device="cuda")
    V = torch.as_tensor(_DeviceRows(v, w.n), device="cuda")
    before = m.copy_data_buffers()
    g = torch.Generator(device="cuda").manual_seed(0)
    h = w.sim.smooth_radius
    # Shifts of up to one cell: most particles change key.
    P[:, :3] += (torch.rand((w.n, 3), device="cuda", generator=g) - 0.5) * (2.0 * h)
    V[:, :3] += 0.25
    torch.cuda.synchronize()
    s = m.copy_data_buffers()
    assert np.abs(s["positions"] - before["positions"]).max() > 0.5 * h
    ids = m.get_ids()
    o = oracle_for(w, m, pos=s["positions"], vel=s["velocities"], ids=ids)
    compare_step(m, o, "device_pointer_edit")
