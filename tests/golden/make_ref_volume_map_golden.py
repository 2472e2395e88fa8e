"""Writes the reference volume-map golden fixtures ``tests/golden/ref_volume_map/*.npz``.

Usage: python tests/golden/make_ref_volume_map_golden.py <path of the VkFluidSim source tree>

Each fixture is one triangle mesh run through the reference's own CPU code: MeshSDF (BVH, angle-
weighted pseudonormals, signed distance at the grid nodes; src/util/mesh_sdf.cpp) with margin
8h and GenerateVolumeMap (16-point Gauss-Legendre over the h-ball; src/util/volume_map.cpp),
compiled by ``oracle/ref_build.py`` against a project-written glm stand-in. A fixture holds the
mesh, h, the resolution and the outputs: grid box, SDF grid and volume map (float, as uploaded).

Only this script (through the recipe) reads the reference tree; tests read the fixtures.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

OUT = HERE / "ref_volume_map"


def icosphere(radius: float, subdivisions: int):
    g = (1 + 5 ** 0.5) / 2
    v = [(-1, g, 0), (1, g, 0), (-1, -g, 0), (1, -g, 0), (0, -1, g), (0, 1, g), (0, -1, -g),
         (0, 1, -g), (g, 0, -1), (g, 0, 1), (-g, 0, -1), (-g, 0, 1)]
    v = [np.array(q, np.float64) / np.linalg.norm(q) for q in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        mid, nf = {}, []
        for a, b, c in f:
            ks = []
            for x, y in ((a, b), (b, c), (c, a)):
                k = (min(x, y), max(x, y))
                if k not in mid:
                    q = v[x] + v[y]
                    v.append(q / np.linalg.norm(q))
                    mid[k] = len(v) - 1
                ks.append(mid[k])
            nf += [(a, ks[0], ks[2]), (b, ks[1], ks[0]), (c, ks[2], ks[1]), tuple(ks)]
        f = nf
    return (np.array(v) * radius).astype(np.float32), np.array(f, np.uint32)


def box(size):
    s = np.asarray(size, np.float32)
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1],
                  [0, 1, 1]], np.float32) * s
    t = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4], [2, 3, 7],
                  [2, 7, 6], [1, 2, 6], [1, 6, 5], [0, 4, 7], [0, 7, 3]], np.uint32)
    return v, t


def l_prism():
    """A non-convex L-shaped prism (its concave edge exercises the edge pseudonormals)."""
    outline = np.array([[0, 0], [0.3, 0], [0.3, 0.1], [0.1, 0.1], [0.1, 0.25], [0, 0.25]], np.float32)
    n = len(outline)
    v = np.concatenate([np.c_[outline, np.zeros(n)], np.c_[outline, np.full(n, 0.12)]]).astype(np.float32)
    tris = []
    for a, b, c in ((0, 1, 2), (0, 2, 3), (0, 3, 4), (0, 4, 5)):  # bottom (z = 0), then top
        tris.append((a, c, b))
        tris.append((a + n, b + n, c + n))
    for k in range(n):  # sides
        a, b = k, (k + 1) % n
        tris.append((a, b, b + n))
        tris.append((a, b + n, a + n))
    return v, np.array(tris, np.uint32)


def cases():
    rng = np.random.default_rng(7)
    v, t = icosphere(0.25, 1)
    bumpy = (v * (1.0 + 0.15 * rng.random((len(v), 1)))).astype(np.float32)
    return {"icosphere": (v, t, 0.04, (20, 20, 20)),
            "box": (*box((0.3, 0.3, 0.3)), 0.05, (16, 18, 20)),
            "l_prism": (*l_prism(), 0.03, (18, 16, 12)),
            "bumpy_sphere": (bumpy, t, 0.035, (18, 18, 18))}


def main(ref: Path):
    from oracle import ref_binding as rb
    from oracle import ref_build

    ref_build.build_volume_map(ref)
    OUT.mkdir(exist_ok=True)
    for name, (v, t, h, res) in cases().items():
        bs, bp, sdf, vm = rb.mesh_volume_map(v, t, h, res)
        np.savez_compressed(OUT / f"{name}.npz", vertices=v, triangles=t, h=np.float32(h),
                            resolution=np.array(res, np.uint32), box_size=bs, box_pos=bp, sdf=sdf,
                            volume_map=vm)
        print(name, len(t), "triangles at", res)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ref_volume_map_golden.py <path of the VkFluidSim "
                 "source tree>")
    main(Path(sys.argv[1]))
