"""Regenerates the golden fixtures of this directory from the VkFluidSim source tree.

Usage: python tests/golden/make_golden.py /path/to/VkFluidSim

* ``gauss_legendre_16.json`` — the 16-point row of the reference's Gauss-Legendre tables
  (src/util/gaussian_quadrature.cpp: weights table from line 8, abscissae table from;
  row n - 2 = 14 of each), read as text. The oracle and the GPU volume-map generator compute
  their own nodes and are checked against these values.
* ``scenes/*.json`` — the reference's two scene fixtures (assets/scenes), verbatim, plus the
  fluid-block particle counts GenericScene::Init derives from them
  (src/scenes/generic_scene.cpp:28-33).

Only this script reads the reference tree; tests read the fixtures it wrote.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _table_rows(text: str, name: str):
    start = text.index(name)
    body = text[text.index("{", start) + 1:]
    rows, depth, cur = [], 0, []
    token = ""
    for ch in body:
        if ch == "{":
            depth += 1
            cur = []
            token = ""
        elif ch == "}":
            if depth == 0:
                break
            if token.strip():
                cur.append(float(token))
            token = ""
            rows.append(cur)
            depth -= 1
        elif ch == "," and depth == 1:
            if token.strip():
                cur.append(float(token))
            token = ""
        elif depth == 1:
            token += ch
    return rows


def main(ref: Path) -> None:
    src = (ref / "src/util/gaussian_quadrature.cpp").read_text()
    src = re.sub(r"//[^\n]*", "", src)
    weights = _table_rows(src, "gauss_legendre_weights")
    points = _table_rows(src, "gauss_legendre_abscissae")
    n = 16
    w16, x16 = weights[n - 2], points[n - 2]
    assert len(w16) == n and len(x16) == n, (len(w16), len(x16))
    (HERE / "gauss_legendre_16.json").write_text(json.dumps(
        {"source": "src/util/gaussian_quadrature.cpp (row n-2 of both tables)", "n": n,
         "abscissae": x16, "weights": w16}, indent=1) + "\n")
    out = HERE / "scenes"
    out.mkdir(exist_ok=True)
    counts = {}
    for name in ("dam_break.json", "obstacle.json"):
        text = (ref / "assets/scenes" / name).read_text()
        (out / name).write_text(text)
        scene = json.loads(text)
        counts[name] = sum(b["size"][0] * b["size"][1] * b["size"][2] for b in scene["fluidBlocks"])
    (out / "expected_counts.json").write_text(json.dumps(counts, indent=1) + "\n")
    print("wrote", sorted(p.name for p in HERE.rglob("*.json")))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the VkFluidSim source tree>")
    main(Path(sys.argv[1]))
