"""CPU tests pinning the FP64 host adjoint used by the GPU adjoint tests: the torch FP64
restatement (tests/fp64_torch_step.py) must reproduce the oracle's FP64 twin rollout, and its
autograd gradients must match FP64 central finite differences (eps 1e-6)."""
from __future__ import annotations

import numpy as np
import pytest

from tests import adjoint_scene as S

torch = pytest.importorskip("torch")
pytest.importorskip("scipy")


@pytest.fixture(scope="module")
def setup():
    w = S.scene()
    return w, S.ObjectList(S.cpu_objects(w))


def _t(v):
    return torch.tensor(v, dtype=torch.float64)


def test_torch_fp64_rollout_reproduces_the_oracle_fp64_twin(setup):
    w, objs = setup
    nu, k = float(w.wcsph.viscosity_strenght), float(w.wcsph.stiffness)
    xo = S.oracle_rollout(w, objs, nu, k, w.vel)
    with torch.no_grad():
        xt = S.torch_rollout(w, objs, _t(nu), _t(k), torch.from_numpy(w.vel.astype(np.float64)))
    travel = np.abs(xo - w.pos).max()
    assert travel > 1e-3
    assert np.abs(xo - xt.numpy()).max() <= 1e-9 * max(1.0, travel)


def test_torch_autograd_matches_fp64_finite_differences(setup):
    w, objs = setup
    tgt = torch.from_numpy(S.target(w))
    nu0, k0 = float(w.wcsph.viscosity_strenght), float(w.wcsph.stiffness)
    v0 = torch.from_numpy(w.vel.astype(np.float64))

    def loss(nu, k, v):
        return ((S.torch_rollout(w, objs, nu, k, v) - tgt) ** 2).mean()

    nu, k, vv = _t(nu0).requires_grad_(True), _t(k0).requires_grad_(True), v0.clone().requires_grad_(True)
    loss(nu, k, vv).backward()
    delta = torch.from_numpy(np.random.default_rng(3).standard_normal(w.vel.shape))
    with torch.no_grad():
        e = 1e-6 * nu0
        fd_nu = (loss(_t(nu0 + e), _t(k0), v0) - loss(_t(nu0 - e), _t(k0), v0)) / (2 * e)
        e = 1e-6 * k0
        fd_k = (loss(_t(nu0), _t(k0 + e), v0) - loss(_t(nu0), _t(k0 - e), v0)) / (2 * e)
        e = 1e-6
        fd_dir = (loss(_t(nu0), _t(k0), v0 + e * delta) - loss(_t(nu0), _t(k0), v0 - e * delta)) / (2 * e)
    assert abs(float(nu.grad) - float(fd_nu)) <= 1e-5 * abs(float(fd_nu))
    assert abs(float(k.grad) - float(fd_k)) <= 1e-5 * abs(float(fd_k))
    assert abs(float((vv.grad * delta).sum()) - float(fd_dir)) <= 1e-5 * abs(float(fd_dir))


def test_adjoint_scenes_cover_both_pair_rules():
    """The GPU adjoint tests' scenes: all keys distinct, mixed, none distinct."""
    frac = {k: float(S.distinct_key_mask(f()).mean()) for k, f in S.SCENES.items()}
    assert frac["one_block"] == 1.0
    assert 0.2 < frac["straddling"] < 0.9
    assert frac["small"] == 0.0
