"""FP64 host restatement of the WCSPH substep in torch, differentiated by autograd: the FP64 host
adjoint the GPU adjoint kernels are checked against (test infrastructure).

It restates the shader passes (assets/shaders/simulation/wcsph_with_boundary_model.slang:102-360)
as order-independent sums over ordered neighbour pairs (i, j) with r_ij <= h, each weighted by the
reference's multiplicity: the number of i's 27 neighbour cells whose key equals j's key (duplicate
keys are walked twice, slang:166-190). Volume-map terms follow CalculateBoundaryVolume with the
clamped grid sampling of the oracle.
"""
from __future__ import annotations

import numpy as np
import torch
from scipy.spatial import cKDTree

M32 = 0xFFFFFFFF


def _hash(c):
    u = (c + 25) & M32
    loc, blk = u % 50, u // 50
    bh = (blk[..., 0] * 15823 + blk[..., 1] * 9737333 + blk[..., 2] * 440817757) & M32
    return (loc[..., 0] + 50 * (loc[..., 1] + 50 * loc[..., 2]) + bh) & M32


OFFS = np.array([[dx, dy, dz] for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)],
                np.int64)


def pairs_with_multiplicity(x: np.ndarray, h: float, n: int):
    """Ordered in-range pairs (i, j), i != j, their multiplicities, and the self multiplicities."""
    cells = np.floor(x / h).astype(np.int64)
    keys = _hash(cells) % n
    nk = _hash(cells[:, None, :] + OFFS[None, :, :]) % n  # (N, 27)
    und = cKDTree(x).query_pairs(h, output_type="ndarray")
    i = np.concatenate([und[:, 0], und[:, 1]])
    j = np.concatenate([und[:, 1], und[:, 0]])
    mult = (nk[i] == keys[j][:, None]).sum(axis=1)
    self_mult = (nk == keys[:, None]).sum(axis=1)
    keep = mult > 0
    return i[keep], j[keep], mult[keep].astype(np.float64), self_mult.astype(np.float64)


def _W(r, P):
    q = r / P["h"]
    s = P["cubic"]
    return torch.where(q <= 1.0, torch.where(q > 0.5, 2.0 * s * (1.0 - q) ** 3,
                                             s * (6.0 * q ** 3 - 6.0 * q ** 2 + 1.0)),
                       torch.zeros_like(r))


def _gw(r, P):
    q = r / P["h"]
    G = P["grad_over_h"]
    val = torch.where(q > 0.5, -G * (1.0 - q) ** 2, G * q * (3.0 * q - 2.0))
    return torch.where((r > 1e-9) & (q <= 1.0), val, torch.zeros_like(r))


def _sample(grid, res, box_pos, box_size, l):
    """Trilinear SampleGrid (slang:51-66) with the cell index clamped to [0, n-2]."""
    chis, cells = [], []
    for a in range(3):
        u = (l[:, a] - box_pos[a]) / box_size[a]
        x = (res[a] - 1.0) * u
        f = torch.clamp(torch.floor(x.detach()), 0.0, float(res[a] - 2))
        cells.append(f.long())
        chis.append(2.0 * (x - f) - 1.0)
    val = 0.0
    for o in range(8):
        ox, oy, oz = o >> 2, o & 1, (o >> 1) & 1
        idx = (cells[0] + ox) + res[0] * ((cells[1] + oy) + res[1] * (cells[2] + oz))
        fac = ((1.0 + (2 * ox - 1) * chis[0]) * (1.0 + (2 * oy - 1) * chis[1]) *
               (1.0 + (2 * oz - 1) * chis[2]))
        val = val + grid[idx] * fac
    return val / 8.0


def boundary_terms(x, P, objs):
    """(Psi, G) of CalculateBoundaryVolume for every particle."""
    n = x.shape[0]
    psi = torch.zeros(n, dtype=x.dtype)
    G = torch.zeros((n, 3), dtype=x.dtype)
    h = P["h"]
    for o in objs:
        T, R = o["T"], o["R"]
        l = x @ T[:3, :3].T + T[:3, 3]
        bp, bs = o["box_pos"], o["box_size"]
        inside = ((l.detach() >= bp) & (l.detach() <= bp + bs)).all(dim=1)
        dist = _sample(o["sdf"], o["res"], bp, bs, l)
        vol = _sample(o["vm"], o["res"], bp, bs, l)
        e = 0.1 * h
        g = []
        for a in range(3):
            d = torch.zeros(3, dtype=x.dtype)
            d[a] = e
            g.append((_sample(o["sdf"], o["res"], bp, bs, l + d) -
                      _sample(o["sdf"], o["res"], bp, bs, l - d)) / (2.0 * e))
        g = torch.stack(g, dim=1)
        modn = torch.sqrt((g * g).sum(dim=1))
        act = inside & (dist.detach() >= 0) & (dist.detach() < h) & (vol.detach() > 0) & \
            (modn.detach() > 1e-9)
        if not bool(act.any()):
            continue
        nrm = (g @ R[:3, :3].T) / modn.clamp_min(1e-30)[:, None]
        d = torch.maximum(dist + 0.125 * h, torch.full_like(dist, 0.5 * h))
        m = act.to(x.dtype)
        psi = psi + m * vol * _W(d, P)
        G = G + (m * vol * _gw(d, P))[:, None] * nrm
    return psi, G


def substep(x, v, P, objs, nu, k):
    """One substep in float64; x, v (N, 3) and nu, k (0-d) are torch tensors."""
    i, j, mult, smult = pairs_with_multiplicity(x.detach().numpy(), P["h"], P["n"])
    i_t, j_t = torch.from_numpy(i), torch.from_numpy(j)
    mu, sm = torch.from_numpy(mult), torch.from_numpy(smult)
    m, rho0, h = P["mass"], P["rho0"], P["h"]
    xij = x[i_t] - x[j_t]
    r = torch.sqrt((xij * xij).sum(dim=1))
    psi, G = boundary_terms(x, P, objs)
    rho = sm * m * _W(torch.zeros_like(sm), P)
    rho = rho.index_add(0, i_t, mu * m * _W(r, P)) + rho0 * psi
    ratio = torch.clamp(rho, min=rho0) / rho0
    p = k * (ratio ** P["expoent"] - 1.0)
    pd = p / (rho * rho)
    pb = p / (rho0 * rho0)
    mr = m / torch.clamp(rho, min=1e-6)
    gw = _gw(r, P)
    nrm = xij / r.clamp_min(1e-30)[:, None]
    Pf = torch.zeros_like(x).index_add(0, i_t, (mu * m * (pd[i_t] + pd[j_t]) * gw)[:, None] * nrm)
    Pf = Pf + ((pd + pb) * rho0)[:, None] * G
    vij = v[i_t] - v[j_t]
    vis = mu * mr[j_t] * (vij * xij).sum(dim=1) * gw / (r * r + 0.01 * h * h)
    Vf = torch.zeros_like(x).index_add(0, i_t, vis[:, None] * nrm)
    lo, hi = P["lo"], P["hi"]
    diff = torch.clamp(x - lo, max=0.0) - torch.clamp(hi - x, max=0.0)
    a = P["g"] - Pf + 10.0 * nu * Vf - P["wall_k"] * diff
    v_new = v + a * P["dt"]
    x_new = x + v_new * P["dt"]
    return x_new, v_new


def params_of(workload):
    """Parameters as the library derives them in double from the float32 fields of the C structs
    (the oracle's FP64 twin does the same)."""
    f = lambda v: float(np.float32(v))  # noqa: E731
    sim, sph, wc = workload.sim, workload.sph, workload.wcsph
    h = f(sim.smooth_radius)
    return {"h": h, "n": workload.n, "cubic": 8.0 / (np.pi * h ** 3),
            "grad_over_h": 48.0 / (np.pi * h ** 4) / h,
            "mass": f(sph.target_density) * (0.8 * h * h * h / 8.0),
            "rho0": f(sph.target_density), "expoent": f(wc.expoent),
            "wall_k": f(wc.wall_stiffness),
            "dt": f(sph.time_scale) * f(sph.fixed_dt) / float(sph.iterations),
            "g": torch.tensor([f(x) for x in sim.gravity], dtype=torch.float64),
            "lo": torch.tensor([f(x) for x in sph.bbox_pos], dtype=torch.float64),
            "hi": torch.tensor([f(a) + f(b) for a, b in zip(sph.bbox_pos, sph.bbox_size)],
                               dtype=torch.float64)}


def objects_of(model):
    out = []
    for k in range(model.n_boundary_objects):
        info = model.get_boundary_object(k)
        T = torch.from_numpy(info.transform.astype(np.float64).reshape(4, 4).T.copy())
        R = torch.from_numpy(info.rotation.astype(np.float64).reshape(4, 4).T.copy())
        out.append({"T": T, "R": R, "box_pos": torch.from_numpy(info.box_pos.astype(np.float64)),
                    "box_size": torch.from_numpy(info.box_size.astype(np.float64)),
                    "res": [int(r) for r in info.resolution],
                    "sdf": torch.from_numpy(info.sdf.astype(np.float64)),
                    "vm": torch.from_numpy(info.volume_map.astype(np.float64))})
    return out
