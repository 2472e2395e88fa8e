"""Runs a checkpointed differentiable rollout of the 65,536-particle dam break (forward + adjoint)
for profilers: ``python -m vkfluidsim_gb300.profile_adjoint --steps 50``."""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import generate_fourier_velocity
from . import workloads as W
from .adjoint import Rollout


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--every", type=int, default=25)
    args = ap.parse_args()
    w = W.dam_break_64k()
    w.vel = generate_fourier_velocity(w.pos, 8, 0.5, 4)
    m = W.build_model(w)
    ro = Rollout(m, args.steps, args.every)
    t0 = time.perf_counter()
    ro.forward()
    xf = ro.final_positions_by_id()
    g = ro.backward(2.0 * (xf - w.pos) / xf.size)
    print(json.dumps({"particles": w.n, "steps": args.steps, "seconds": time.perf_counter() - t0,
                      "dnu": g["dnu"], "dk": g["dk"], "dv0_max": float(np.abs(g["dv0"]).max())}))


if __name__ == "__main__":
    main()
