"""The rule that lets a skin-list build skip duplicate buckets, restated on the host and checked
against brute force (the CUDA function is skin_keys_distinct in vkfluidsim_gb300/csrc/vfs_kernels.cu;
the GPU tests check the kernels that use it against the oracle).

HashCell3D (spatial_hash_3d.slang:16-32) is linear inside a 50^3 block of cells. A particle's list
is built only when the rule proves the 125 keys of its 5x5x5 block of cells distinct; a claim of
"distinct" must never be wrong, and away from the 2^32 wrap of the hashes it is exact."""
from __future__ import annotations

import numpy as np
import pytest

M = 0xFFFFFFFF


def hash_cell(x, y, z):
    """HashCell3D(cell) as uint arithmetic (spatial_hash_3d.slang:16-27)."""
    ux, uy, uz = (x + 25) & M, (y + 25) & M, (z + 25) & M
    loc = (ux % 50, uy % 50, uz % 50)
    blk = (ux // 50, uy // 50, uz // 50)
    bh = (blk[0] * 15823 + blk[1] * 9737333 + blk[2] * 440817757) & M
    return (loc[0] + 50 * (loc[1] + 50 * loc[2]) + bh) & M


def first_block_cells(c):
    b0 = ((c - 2 + 25) & M) // 50
    return 1 + sum(1 for t in range(1, 5) if ((c - 2 + t + 25) & M) // 50 == b0)


def boxes_share_a_key(ka, wa, kb, wb, n):
    """Does a key (ka + x + 50 y + 2500 z) mod n of box a equal one of box b's? (b's keys are
    kb + its offsets; an offset's base-50 / 2500 digits lie below b's widths.)"""
    for z in range(wa[2]):
        for y in range(wa[1]):
            for x in range(wa[0]):
                d = ((ka + x + 50 * y + 2500 * z) % n - kb) % n
                oz, r = divmod(d, 2500)
                oy, ox = divmod(r, 50)
                if ox < wb[0] and oy < wb[1] and oz < wb[2]:
                    return True
    return False


def keys_distinct(n, cx, cy, cz):
    """The rule: split the 5x5x5 block into its per-hash-block boxes; each box's keys lie in a
    circular interval [hmin mod n, hmin mod n + span]; with n > 10204 and no box's hashes
    wrapping 2^32, boxes whose intervals are disjoint modulo n share no key, and boxes whose
    intervals overlap are compared key by key."""
    if n <= 10204:
        return False
    fx, fy, fz = first_block_cells(cx), first_block_cells(cy), first_block_cells(cz)
    ks, spans, widths = [], [], []
    for bz in range(2 if fz < 5 else 1):
        for by in range(2 if fy < 5 else 1):
            for bx in range(2 if fx < 5 else 1):
                x0, x1 = (fx, 4) if bx else (0, fx - 1)
                y0, y1 = (fy, 4) if by else (0, fy - 1)
                z0, z1 = (fz, 4) if bz else (0, fz - 1)
                lo = hash_cell(cx - 2 + x0, cy - 2 + y0, cz - 2 + z0)
                hi = hash_cell(cx - 2 + x1, cy - 2 + y1, cz - 2 + z1)
                if hi < lo:
                    return False
                ks.append(lo % n)
                spans.append(hi - lo)
                widths.append((x1 - x0 + 1, y1 - y0 + 1, z1 - z0 + 1))
    for a in range(1, len(ks)):
        for b in range(a):
            if ((ks[b] - ks[a]) % n <= spans[a] or (ks[a] - ks[b]) % n <= spans[b]) and \
                    boxes_share_a_key(ks[a], widths[a], ks[b], widths[b], n):
                return False
    return True


def brute_distinct(n, cx, cy, cz):
    keys = {hash_cell((cx + dx) & M, (cy + dy) & M, (cz + dz) & M) % n
            for dx in range(-2, 3) for dy in range(-2, 3) for dz in range(-2, 3)}
    return len(keys) == 125


@pytest.mark.parametrize("region", ["boundaries", "wrap", "far"])
def test_rule_never_claims_a_duplicate(region):
    rng = np.random.default_rng({"boundaries": 0, "wrap": 1, "far": 2}[region])
    claims = 0
    for trial in range(2500):
        n = int(rng.choice([10205, 12345, 20000, 65536, 1048576, 4613734]))
        if region == "boundaries":  # cells around the 50-cell block faces
            c = rng.integers(-60, 200, 3)
        elif region == "wrap":  # cells whose cell + 25 wraps 2^32
            c = rng.integers(-30, -20, 3)
        else:
            c = rng.integers(0, 100000, 3)
        cx, cy, cz = (int(v) & M for v in c)
        if keys_distinct(n, cx, cy, cz):
            claims += 1
            assert brute_distinct(n, cx, cy, cz), (n, cx, cy, cz)
        elif region != "wrap":  # away from the 2^32 wrap of the hashes the rule is exact
            assert not brute_distinct(n, cx, cy, cz), (n, cx, cy, cz)
    assert claims > 0


def test_small_scenes_are_never_claimed():
    for cx in range(0, 60, 7):
        assert not keys_distinct(10204, cx, 3, 4)


def test_rule_covers_most_particles_of_the_1m_scene():
    """Every particle of the 1M obstacle scene's initial state gets a list (99.2% did when boxes
    with overlapping key intervals were refused without comparing their keys; 77% would if the
    whole block had to lie in one hash block)."""
    from vkfluidsim_gb300 import workloads as W

    w = W.obstacle_1m(seed=1)
    c = np.floor(w.pos / np.float32(w.sim.smooth_radius)).astype(np.int64)
    cells, inverse = np.unique(c, axis=0, return_inverse=True)
    ok = np.array([keys_distinct(w.n, int(x) & M, int(y) & M, int(z) & M) for x, y, z in cells])
    frac = ok[inverse.ravel()].mean()
    assert frac == 1.0, frac
