"""FP64 restatement of a long WCSPH rollout in torch, on any device, for the gradient checks at the
differentiable benchmark's own scale (65,536 particles, 300 substeps, checkpoint every 25).
Test infrastructure, like tests/fp64_torch_step.py, whose kernel functions and multiplicity rule it
reuses (assets/shaders/simulation/wcsph_with_boundary_model.slang:153-360: every in-range ordered
pair (i, j), i != j, weighted by the number of i's 27 neighbour cells whose key equals j's key).

Scenes without boundary objects only (walls by the reference's penalty force). It shares nothing
with the GPU path under test: the candidate pairs come from a k-d tree on the host, and every sum
is an order-independent index_add in float64.

* Candidate pairs are found once per checkpoint segment within h + skin (a k-d tree on the host);
  every substep keeps those within h with positive multiplicity. A pair within h at some substep
  of the segment is a candidate as long as no particle moves skin / 2 within the segment, which
  is checked at the end of every segment (the rollout raises otherwise).
* With grad=True each segment runs under torch.utils.checkpoint, so autograd keeps one segment's
  graph at a time and recomputes the others (the same candidates: they depend on the segment's
  start only).
"""
from __future__ import annotations

import numpy as np
import torch
from scipy.spatial import cKDTree
from torch.utils.checkpoint import checkpoint

from tests.fp64_torch_step import OFFS, _gw, _W

M32 = 0xFFFFFFFF


def _hash_t(c):
    u = (c + 25) & M32
    loc, blk = u % 50, u // 50
    bh = (blk[..., 0] * 15823 + blk[..., 1] * 9737333 + blk[..., 2] * 440817757) & M32
    return (loc[..., 0] + 50 * (loc[..., 1] + 50 * loc[..., 2]) + bh) & M32


def params_of(w, device):
    """Parameters from the float32 fields of the C structs, in double (as the library derives
    them)."""
    f = lambda v: float(np.float32(v))  # noqa: E731
    sim, sph, wc = w.sim, w.sph, w.wcsph
    h = f(sim.smooth_radius)
    t = lambda a: torch.tensor(a, dtype=torch.float64, device=device)  # noqa: E731
    return {"h": h, "n": w.n, "cubic": 8.0 / (np.pi * h ** 3),
            "grad_over_h": 48.0 / (np.pi * h ** 4) / h,
            "mass": f(sph.target_density) * (0.8 * h * h * h / 8.0),
            "rho0": f(sph.target_density), "expoent": f(wc.expoent), "wall_k": f(wc.wall_stiffness),
            "dt": f(sph.time_scale) * f(sph.fixed_dt) / float(sph.iterations),
            "g": t([f(x) for x in sim.gravity]), "lo": t([f(x) for x in sph.bbox_pos]),
            "hi": t([f(a) + f(b) for a, b in zip(sph.bbox_pos, sph.bbox_size)]),
            "offs": torch.from_numpy(OFFS).to(device)}


def candidates(x: torch.Tensor, radius: float):
    """Ordered pairs (i, j), i != j, within `radius` (k-d tree on the host)."""
    und = cKDTree(x.detach().cpu().numpy()).query_pairs(radius, output_type="ndarray")
    i = np.concatenate([und[:, 0], und[:, 1]])
    j = np.concatenate([und[:, 1], und[:, 0]])
    return torch.from_numpy(i).to(x.device), torch.from_numpy(j).to(x.device)


def substep(x, v, P, nu, k, cand):
    h, n = P["h"], P["n"]
    ci, cj = cand
    with torch.no_grad():
        cells = torch.floor(x / h).long()
        keys = _hash_t(cells) % n
        nk = _hash_t(cells[:, None, :] + P["offs"][None, :, :]) % n  # (N, 27)
        d = x[ci] - x[cj]
        inr = (d * d).sum(dim=1) <= h * h
        ci, cj = ci[inr], cj[inr]
        mult = (nk[ci] == keys[cj][:, None]).sum(dim=1)
        keep = mult > 0
        i_t, j_t, mu = ci[keep], cj[keep], mult[keep].to(torch.float64)
        sm = (nk == keys[:, None]).sum(dim=1).to(torch.float64)
    m, rho0 = P["mass"], P["rho0"]
    xij = x[i_t] - x[j_t]
    r = torch.sqrt((xij * xij).sum(dim=1))
    rho = sm * m * _W(torch.zeros_like(sm), P)
    rho = rho.index_add(0, i_t, mu * m * _W(r, P))
    p = k * ((torch.clamp(rho, min=rho0) / rho0) ** P["expoent"] - 1.0)
    pd = p / (rho * rho)
    mr = m / torch.clamp(rho, min=1e-6)
    gw = _gw(r, P)
    nrm = xij / r.clamp_min(1e-30)[:, None]
    Pf = torch.zeros_like(x).index_add(0, i_t, (mu * m * (pd[i_t] + pd[j_t]) * gw)[:, None] * nrm)
    vij = v[i_t] - v[j_t]
    vis = mu * mr[j_t] * (vij * xij).sum(dim=1) * gw / (r * r + 0.01 * h * h)
    Vf = torch.zeros_like(x).index_add(0, i_t, vis[:, None] * nrm)
    diff = torch.clamp(x - P["lo"], max=0.0) - torch.clamp(P["hi"] - x, max=0.0)
    a = P["g"] - Pf + 10.0 * nu * Vf - P["wall_k"] * diff
    v_new = v + a * P["dt"]
    return x + v_new * P["dt"], v_new


def rollout(w, nu, k, v0, steps: int, every: int = 25, skin: float = 0.02, grad: bool = False,
            device="cuda"):
    """Final positions (by id, float64 tensor on `device`) of the FP64 rollout of workload `w`
    (no boundary objects) with viscosity nu, stiffness k (0-d tensors) and initial velocity v0
    ((N, 3) tensor)."""
    if w.objects:
        raise ValueError("the FP64 rollout restates scenes without boundary objects only")
    P = params_of(w, device)
    x = torch.from_numpy(w.pos.astype(np.float64)).to(device)
    v = v0
    done = 0
    while done < steps:
        count = min(every, steps - done)
        cand = candidates(x, P["h"] + skin)
        x_start = x.detach()

        def seg(x_, v_, nu_, k_, cand=cand, count=count):
            for _ in range(count):
                x_, v_ = substep(x_, v_, P, nu_, k_, cand)
            return x_, v_

        if grad:
            x, v = checkpoint(seg, x, v, nu, k, use_reentrant=False)
        else:
            x, v = seg(x, v, nu, k)
        moved = float(torch.sqrt(((x.detach() - x_start) ** 2).sum(dim=1)).max())
        if moved >= 0.5 * skin:
            raise RuntimeError(f"a particle moved {moved:.3g} m in one segment (skin {skin})")
        done += count
    return x
