"""Spatial-hash compute primitives on device buffers, mirroring the reference's
``GPUCountSort::Run``, ``SpatialOffset::Run`` and ``BufferReorder`` (src/compute/sort.h:152-234).

Arguments are device pointers (ints; e.g. ``torch.Tensor.data_ptr()``) and an optional CUDA stream
handle; the calls enqueue work and return without synchronising.
"""
from __future__ import annotations

import ctypes as C

from ._abi import check, load_library


def sort_pairs(items_ptr: int, keys_ptr: int, n: int, max_value: int, stream: int = 0) -> None:
    """Stable in-place sort of (key, item) pairs; items become the sorting permutation."""
    check(load_library().vfs_sort_pairs(C.c_void_p(items_ptr), C.c_void_p(keys_ptr), n, max_value,
                                        C.c_void_p(stream)))


def sort_status(stream: int = 0) -> int:
    """Synchronises the stream and returns (then clears) the error bits of the pair sorts run
    since the last call; raises VfsError (VFS_ERR_DEVICE_CHECK) when a sort's look-back timed
    out."""
    err = C.c_uint32(0)
    check(load_library().vfs_sort_pairs_status(C.c_void_p(stream), C.byref(err)))
    return int(err.value)


def spatial_offsets(sorted_keys_ptr: int, offsets_ptr: int, n: int, stream: int = 0) -> None:
    """offsets[k] = first index of key k in the sorted keys, n for absent keys."""
    check(load_library().vfs_spatial_offsets(C.c_void_p(sorted_keys_ptr), C.c_void_p(offsets_ptr),
                                             n, C.c_void_p(stream)))


def reorder_float3(sorted_indices_ptr: int, src_ptr: int, dst_ptr: int, n: int,
                   stream: int = 0) -> None:
    """dst[i] = src[sorted_indices[i]] for packed float3 arrays."""
    check(load_library().vfs_reorder_float3(C.c_void_p(sorted_indices_ptr), C.c_void_p(src_ptr),
                                            C.c_void_p(dst_ptr), n, C.c_void_p(stream)))
