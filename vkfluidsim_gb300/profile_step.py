"""Runs a few WCSPH substeps of a named workload with one kernel launch per pass (no CUDA graph),
for profilers: ``python -m vkfluidsim_gb300.profile_step --workload obstacle_1m --substeps 3``.
Prints the per-pass event times of the last substeps."""
from __future__ import annotations

import argparse
import json

from . import workloads as W


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="obstacle_1m", choices=sorted(W.WORKLOADS))
    ap.add_argument("--substeps", type=int, default=3)
    ap.add_argument("--digits", type=int, default=0)
    ap.add_argument("--tile-items", type=int, default=16)
    args = ap.parse_args()
    w = W.WORKLOADS[args.workload]()
    m = W.build_model(w)
    if args.digits:
        m.set_sort_config(args.digits, args.tile_items)
    m.use_graph(False)
    m.substeps(1)
    prof = m.profile_substeps(max(1, args.substeps - 1))
    m.synchronize()
    print(json.dumps({"workload": w.name, "particles": w.n, "phase_ms": prof,
                      "sort": m.get_sort_config()}))


if __name__ == "__main__":
    main()
