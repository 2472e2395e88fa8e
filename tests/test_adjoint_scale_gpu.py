"""Gradient checks of the differentiable rollout at the differentiable benchmark's own scale:
65,536 particles, 300 substeps, checkpoint every 25 (vkfluidsim_gb300.workloads.dam_break_64k).

The target is the rollout with viscosity 0.02, stiffness 60 and a smooth initial velocity (8
Fourier modes, 0.5 m/s); the differentiated run starts from viscosity 0.01, stiffness 50 and zero
velocity; loss = mean squared error of the final positions by id (as bench.py's fwd_adjoint leg).
The GPU adjoint's gradients with respect to viscosity, stiffness and the initial velocity field
are compared with an FP64 host adjoint (tests/fp64_torch_rollout.py under torch autograd, run in
float64 on the GPU as a checker) on the benchmark scene itself, and with FP64 central finite
differences (eps 1e-6 relative for the parameters, 1e-6 along a random unit-scale direction of
the velocity field) on the same scene moved into one 50^3 hash block, where every particle's 27
neighbour keys are distinct during the whole rollout, so the loss is smooth in its inputs.
Bar: 1e-3 relative (normwise for the velocity field). All 300 substeps are used.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from tests.helpers import normwise_rel
from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
pytest.importorskip("scipy")

TOL = 1e-3
STEPS, EVERY = 300, 25
SHIFT = np.array([-0.9, -0.45, -0.45], np.float32)  # into hash block 0 (cells -25..24)


def _shifted(w):
    w = replace(w, pos=(w.pos + SHIFT).astype(np.float32),
                sph=replace(w.sph, bbox_pos=tuple(float(a + b) for a, b in zip(w.sph.bbox_pos, SHIFT))))
    return w


def _gpu_case(base):
    """Target positions and the GPU adjoint's gradients at (nu 0.01, k 50, v0 = 0)."""
    from vkfluidsim_gb300.adjoint import Rollout

    tw = replace(base, vel=vfs.generate_fourier_velocity(base.pos, 8, 0.5, 4),
                 wcsph=replace(base.wcsph, viscosity_strenght=0.02, stiffness=60.0))
    tm = W.build_model(tw)
    tm.substeps(STEPS)
    ts = tm.copy_data_buffers()
    target = np.empty_like(ts["positions"])
    target[tm.get_ids()] = ts["positions"]
    del tm
    m = W.build_model(base)
    ro = Rollout(m, STEPS, EVERY)
    ro.forward()
    xf = ro.final_positions_by_id()
    g = ro.backward(2.0 * (xf - target) / xf.size)
    return target.astype(np.float64), g, float(np.mean((xf.astype(np.float64) - target) ** 2))


def _t(v):
    return torch.tensor(v, dtype=torch.float64, device="cuda")


def _host_grads(w, target):
    from tests import fp64_torch_rollout as R

    tgt = torch.from_numpy(target).cuda()
    nu = _t(float(w.wcsph.viscosity_strenght)).requires_grad_(True)
    k = _t(float(w.wcsph.stiffness)).requires_grad_(True)
    v0 = torch.zeros((w.n, 3), dtype=torch.float64, device="cuda", requires_grad=True)
    loss = ((R.rollout(w, nu, k, v0, STEPS, EVERY, grad=True) - tgt) ** 2).mean()
    loss.backward()
    return {"loss": float(loss.detach()), "dnu": float(nu.grad), "dk": float(k.grad),
            "dv0": v0.grad.cpu().numpy()}


def _report(label, g, h):
    print(f"{label}: d/dnu gpu {g['dnu']:.8g} fp64 {h['dnu']:.8g} | d/dk gpu {g['dk']:.8g} "
          f"fp64 {h['dk']:.8g} | dv0 normwise {normwise_rel(g['dv0'], h['dv0']):.3g}")


def test_config4_adjoint_matches_the_fp64_host_adjoint():
    base = W.dam_break_64k()
    assert (base.n, base.steps) == (65536, STEPS) and not base.objects
    target, g, loss_gpu = _gpu_case(base)
    h = _host_grads(base, target)
    print(f"loss gpu {loss_gpu:.8g} fp64 {h['loss']:.8g}")
    _report("dam_break_64k, 300 substeps", g, h)
    assert abs(g["dnu"] - h["dnu"]) <= TOL * abs(h["dnu"])
    assert abs(g["dk"] - h["dk"]) <= TOL * abs(h["dk"])
    assert normwise_rel(g["dv0"], h["dv0"]) <= TOL


def test_config4_gradients_match_fp64_finite_differences():
    from tests import fp64_torch_rollout as R
    from tests.adjoint_scene import distinct_key_mask

    w = _shifted(W.dam_break_64k())
    assert distinct_key_mask(w).all()
    target, g, _ = _gpu_case(w)
    h = _host_grads(w, target)
    _report("dam_break_64k moved into one hash block", g, h)
    tgt = torch.from_numpy(target).cuda()
    nu0, k0 = float(w.wcsph.viscosity_strenght), float(w.wcsph.stiffness)
    z = torch.zeros((w.n, 3), dtype=torch.float64, device="cuda")
    delta = np.random.default_rng(3).standard_normal((w.n, 3))
    dt = torch.from_numpy(delta).cuda()

    def loss(nu, k, v0):
        x = R.rollout(w, _t(nu), _t(k), v0, STEPS, EVERY)
        # All 27 neighbour keys stay distinct through the rollout.
        assert distinct_key_mask(replace(w, pos=x.cpu().numpy().astype(np.float32))).all()
        return float(((x - tgt) ** 2).mean())

    with torch.no_grad():
        e = 1e-6 * nu0
        fd_nu = (loss(nu0 + e, k0, z) - loss(nu0 - e, k0, z)) / (2 * e)
        e = 1e-6 * k0
        fd_k = (loss(nu0, k0 + e, z) - loss(nu0, k0 - e, z)) / (2 * e)
        e = 1e-6
        fd_dir = (loss(nu0, k0, e * dt) - loss(nu0, k0, -e * dt)) / (2 * e)
    gpu_dir = float(np.sum(g["dv0"].astype(np.float64) * delta))
    host_dir = float(np.sum(h["dv0"] * delta))
    print(f"FD d/dnu {fd_nu:.8g} gpu {g['dnu']:.8g} | FD d/dk {fd_k:.8g} gpu {g['dk']:.8g} | "
          f"FD dir {fd_dir:.8g} gpu {gpu_dir:.8g} fp64 adjoint {host_dir:.8g}")
    for gpu, host, fd in ((g["dnu"], h["dnu"], fd_nu), (g["dk"], h["dk"], fd_k),
                          (gpu_dir, host_dir, fd_dir)):
        assert abs(host - fd) <= TOL * abs(fd)
        assert abs(gpu - fd) <= TOL * abs(fd)
    assert normwise_rel(g["dv0"], h["dv0"]) <= TOL
