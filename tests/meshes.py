"""Triangle meshes for the mesh-object tests (generated here, outward-facing triangles)."""
from __future__ import annotations

import numpy as np


def box(half=(0.5, 0.5, 0.5)):
    """The 12-triangle box [-half, half]."""
    hx, hy, hz = half
    v = np.array([[x, y, z] for z in (-hz, hz) for y in (-hy, hy) for x in (-hx, hx)], np.float32)
    # Vertex index = x + 2 y + 4 z (bits); faces as quads with outward counter-clockwise winding.
    quads = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    t = []
    for a, b, c, d in quads:
        t += [(a, b, c), (a, c, d)]
    return v, np.array(t, np.uint32)


def icosphere(radius=0.3, subdivisions=1):
    """A subdivided icosahedron projected onto the sphere."""
    g = (1 + 5 ** 0.5) / 2
    v = [(-1, g, 0), (1, g, 0), (-1, -g, 0), (1, -g, 0), (0, -1, g), (0, 1, g), (0, -1, -g),
         (0, 1, -g), (g, 0, -1), (g, 0, 1), (-g, 0, -1), (-g, 0, 1)]
    v = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        mid = {}

        def m(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                p = v[a] + v[b]
                v.append(p / np.linalg.norm(p))
                mid[k] = len(v) - 1
            return mid[k]

        nf = []
        for a, b, c in f:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return (np.array(v) * radius).astype(np.float32), np.array(f, np.uint32)


def write_obj(path, v, t, extra_object_first=False):
    lines = []
    if extra_object_first:  # a decoy object: the loader takes the file's last object
        lines += ["o decoy", "v 9 9 9", "v 9 9.5 9", "v 9.5 9 9", "f 1 2 3"]
        off = 3
    else:
        off = 0
    lines.append("o mesh")
    lines += [f"v {x:.9g} {y:.9g} {z:.9g}" for x, y, z in v]
    lines += [f"f {a + 1 + off}/1 {b + 1 + off}/1 {c + 1 + off}/1" for a, b, c in t]
    path.write_text("\n".join(lines) + "\n")
