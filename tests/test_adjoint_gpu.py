"""GPU tests of the differentiable rollout (the C ABI's checkpointed adjoint).

Loss: mean squared error of the final positions (by particle id) against a target. Gradients with
respect to viscosity, stiffness and the initial velocity field are checked against the FP64 host
adjoint (tests/fp64_torch_step.py under torch autograd, itself pinned to the oracle's FP64 twin and
to FP64 central finite differences in tests/test_fp64_reference.py) and against FP64 central
finite differences (eps 1e-6) of that FP64 rollout. Bar: 1e-3 relative (normwise for the
per-particle field).

Three scenes cover the adjoint's pair rules: all particles with distinct neighbour keys (pair
terms gathered), a lattice straddling a hash-block boundary (gathered and scattered terms mixed)
and a scene of 1,440 particles (every pair term scattered, duplicate neighbour keys present).
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import adjoint_scene as S
from tests.helpers import normwise_rel
from vkfluidsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
pytest.importorskip("scipy")

TOL = 1e-3


def _t(v):
    return torch.tensor(v, dtype=torch.float64)


@pytest.fixture(scope="module", params=sorted(S.SCENES))
def gpu_grads(request):
    from vkfluidsim_gb300.adjoint import Rollout

    w = S.SCENES[request.param]()
    m = W.build_model(w)
    ro = Rollout(m, S.STEPS, S.EVERY)
    ro.forward()
    xf = ro.final_positions_by_id().astype(np.float64)
    target = S.target(w)
    g = ro.backward(2.0 * (xf - target) / xf.size)
    return w, m, target, g


@pytest.fixture(scope="module")
def host_grads(gpu_grads):
    w, m, target, _ = gpu_grads
    tgt = torch.from_numpy(target)
    nu0, k0 = float(w.wcsph.viscosity_strenght), float(w.wcsph.stiffness)
    v0 = torch.from_numpy(w.vel.astype(np.float64))

    def loss(nu, k, v):
        return ((S.torch_rollout(w, m, nu, k, v) - tgt) ** 2).mean()

    nu, k, vv = _t(nu0).requires_grad_(True), _t(k0).requires_grad_(True), v0.clone().requires_grad_(True)
    loss(nu, k, vv).backward()
    out = {"dnu": float(nu.grad), "dk": float(k.grad), "dv0": vv.grad.numpy(), "loss": loss}
    if S.distinct_key_mask(w).all():
        # Finite differences only where no neighbour multiplicity can change under a perturbation.
        delta = np.random.default_rng(3).standard_normal(w.vel.shape)
        dt = torch.from_numpy(delta)
        with torch.no_grad():
            e = 1e-6 * nu0
            fd_nu = float((loss(_t(nu0 + e), _t(k0), v0) - loss(_t(nu0 - e), _t(k0), v0)) / (2 * e))
            e = 1e-6 * k0
            fd_k = float((loss(_t(nu0), _t(k0 + e), v0) - loss(_t(nu0), _t(k0 - e), v0)) / (2 * e))
            e = 1e-6
            fd_dir = float((loss(_t(nu0), _t(k0), v0 + e * dt) - loss(_t(nu0), _t(k0), v0 - e * dt))
                           / (2 * e))
        out.update(fd_nu=fd_nu, fd_k=fd_k, fd_dir=fd_dir, delta=delta)
    return out


def test_rollout_forward_matches_plain_stepping(gpu_grads):
    w, m, target, g = gpu_grads
    m2 = W.build_model(w)
    m2.substeps(S.STEPS)
    s2, s1 = m2.copy_data_buffers(), m.copy_data_buffers()  # the rollout ends at its final state
    x2 = np.empty_like(s2["positions"])
    x2[m2.get_ids()] = s2["positions"]
    x1 = np.empty_like(s1["positions"])
    x1[m.get_ids()] = s1["positions"]
    assert np.array_equal(x1, x2)


def test_adjoint_matches_the_fp64_host_adjoint(gpu_grads, host_grads):
    _, _, _, g = gpu_grads
    h = host_grads
    print("d/dnu gpu", g["dnu"], "fp64", h["dnu"], "| d/dk gpu", g["dk"], "fp64", h["dk"],
          "| dv0 normwise", normwise_rel(g["dv0"], h["dv0"]))
    assert abs(g["dnu"] - h["dnu"]) <= TOL * abs(h["dnu"])
    assert abs(g["dk"] - h["dk"]) <= TOL * abs(h["dk"])
    assert normwise_rel(g["dv0"], h["dv0"]) <= TOL


def test_adjoint_matches_fp64_finite_differences(gpu_grads, host_grads):
    _, _, _, g = gpu_grads
    h = host_grads
    if "fd_nu" not in h:
        pytest.skip("finite differences only on the scene whose neighbour keys are all distinct")
    gpu_dir = float(np.sum(g["dv0"].astype(np.float64) * h["delta"]))
    print("FD d/dnu", h["fd_nu"], "gpu", g["dnu"], "| FD d/dk", h["fd_k"], "gpu", g["dk"],
          "| FD dir", h["fd_dir"], "gpu", gpu_dir)
    assert abs(g["dnu"] - h["fd_nu"]) <= TOL * abs(h["fd_nu"])
    assert abs(g["dk"] - h["fd_k"]) <= TOL * abs(h["fd_k"])
    assert abs(gpu_dir - h["fd_dir"]) <= TOL * abs(h["fd_dir"])


def test_autograd_function_wraps_the_adjoint(gpu_grads):
    from vkfluidsim_gb300.adjoint import rollout_function

    w, m, target, g = gpu_grads
    if w.n != S.scene().n or not S.distinct_key_mask(w).all():
        pytest.skip("checked on the first scene")
    fn = rollout_function()
    v0 = torch.from_numpy(w.vel.astype(np.float32)).requires_grad_(True)
    nu = torch.tensor(float(w.wcsph.viscosity_strenght), requires_grad=True)
    k = torch.tensor(float(w.wcsph.stiffness), requires_grad=True)
    xf = fn.apply(v0, nu, k, w, S.STEPS, S.EVERY)
    loss = ((xf.double() - torch.from_numpy(target)) ** 2).mean()
    loss.backward()
    assert abs(float(nu.grad) - g["dnu"]) <= 1e-4 * abs(g["dnu"])
    assert abs(float(k.grad) - g["dk"]) <= 1e-4 * abs(g["dk"])
    assert normwise_rel(v0.grad.numpy(), g["dv0"]) <= 1e-4


def test_backward_repeats_without_and_with_a_new_forward():
    """A second backward recomputes the last segment (the forward pass recorded it); a new forward
    from the same state gives the same gradients again (up to atomic summation order)."""
    from vkfluidsim_gb300.adjoint import Rollout

    w = S.scene()
    m = W.build_model(w)
    ro = Rollout(m, S.STEPS, S.EVERY)
    ro.forward()
    xf = ro.final_positions_by_id()
    seed = 2.0 * (xf - S.target(w)) / xf.size
    g1 = ro.backward(seed)
    g2 = ro.backward(seed)
    m.set_particle_state(w.pos, w.vel)
    ro.forward()
    assert np.array_equal(ro.final_positions_by_id(), xf)
    g3 = ro.backward(seed)
    for g in (g2, g3):
        assert abs(g["dnu"] - g1["dnu"]) <= 1e-5 * abs(g1["dnu"])
        assert abs(g["dk"] - g1["dk"]) <= 1e-5 * abs(g1["dk"])
        assert normwise_rel(g["dv0"], g1["dv0"]) <= 1e-5
