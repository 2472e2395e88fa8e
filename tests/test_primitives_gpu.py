"""GPU tests of the standalone compute primitives (GPUCountSort::Run, SpatialOffset::Run,
BufferReorder) through the C ABI, against numpy restatements of the reference semantics."""
from __future__ import annotations

import numpy as np
import pytest

from vkfluidsim_gb300 import primitives as P

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("n,max_value", [(1, 0), (7, 3), (4097, 4096), (100_000, 99_999),
                                         (300_000, 1023), (1 << 20, (1 << 20) - 1),
                                         (50_000, 2**32 - 1)])
def test_sort_pairs_is_the_stable_counting_sort(n, max_value):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, max_value + 1, size=n, dtype=np.uint64).astype(np.uint32)
    k = _dev(keys.view(np.int32))
    items = torch.full((n,), 12345, dtype=torch.int32, device="cuda")
    P.sort_pairs(items.data_ptr(), k.data_ptr(), n, max_value)
    torch.cuda.synchronize()
    assert P.sort_status() == 0  # no look-back timed out
    perm = np.argsort(keys, kind="stable").astype(np.uint32)
    assert np.array_equal(items.cpu().numpy().view(np.uint32), perm)
    assert np.array_equal(k.cpu().numpy().view(np.uint32), keys[perm])


def test_spatial_offsets_and_reorder():
    n = 70_000
    rng = np.random.default_rng(1)
    keys = np.sort(rng.integers(0, n, size=n).astype(np.uint32))
    offs = torch.empty(n, dtype=torch.int32, device="cuda")
    P.spatial_offsets(_dev(keys.view(np.int32)).data_ptr(), offs.data_ptr(), n)
    first = np.full(n, n, np.uint32)
    for i in range(n - 1, -1, -1):
        first[keys[i]] = i
    torch.cuda.synchronize()
    assert np.array_equal(offs.cpu().numpy().view(np.uint32), first)
    idx = rng.permutation(n).astype(np.uint32)
    src = rng.random((n, 3)).astype(np.float32)
    d_idx, d_src = _dev(idx.view(np.int32)), _dev(src)
    dst = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    P.reorder_float3(d_idx.data_ptr(), d_src.data_ptr(), dst.data_ptr(), n)
    torch.cuda.synchronize()
    assert np.array_equal(dst.cpu().numpy(), src[idx])
