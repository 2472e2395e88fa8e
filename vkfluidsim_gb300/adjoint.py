"""Differentiable rollouts: the C ABI's checkpointed forward/adjoint (vfs_rollout_*) and a
``torch.autograd.Function`` over it.

Gradients are returned by particle id (the order in which the state was first set). The loss of the
65,536-particle differentiable benchmark workload is the mean squared error of the final
positions by id.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import replace

import numpy as np

from . import workloads as W
from ._abi import check, load_library
from .model import _fp


class Rollout:
    """A checkpointed differentiable rollout of `model` from its current state."""

    def __init__(self, model, steps: int, checkpoint_every: int = 25):
        self._lib = load_library()
        self.model = model
        self.n = model.n_particles
        h = C.c_void_p()
        check(self._lib.vfs_rollout_create(model._h, steps, checkpoint_every, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.vfs_rollout_destroy(self._h)
            self._h = C.c_void_p()

    def forward(self) -> None:
        check(self._lib.vfs_rollout_forward(self._h))

    def final_positions_by_id(self) -> np.ndarray:
        s = self.model.copy_data_buffers()
        out = np.empty_like(s["positions"])
        out[self.model.get_ids()] = s["positions"]
        return out

    def backward(self, dl_dx_final, dl_dv_final=None) -> dict:
        gx = None if dl_dx_final is None else np.ascontiguousarray(dl_dx_final, np.float32).reshape(-1, 3)
        gv = None if dl_dv_final is None else np.ascontiguousarray(dl_dv_final, np.float32).reshape(-1, 3)
        dv0 = np.empty((self.n, 3), np.float32)
        dx0 = np.empty((self.n, 3), np.float32)
        dp = (C.c_double * 2)()
        check(self._lib.vfs_rollout_backward(self._h, _fp(gx), _fp(gv), _fp(dv0), _fp(dx0), dp))
        return {"dv0": dv0, "dx0": dx0, "dnu": float(dp[0]), "dk": float(dp[1])}


def rollout_function():
    """Returns a torch.autograd.Function computing final positions (by id) of a workload rolled
    out from initial velocities v0 with viscosity nu and stiffness k; its backward runs the GPU
    adjoint. torch is imported lazily (it is only needed for this wrapper)."""
    import torch

    class WCSPHRollout(torch.autograd.Function):
        @staticmethod
        def forward(ctx, v0, nu, k, workload, steps, checkpoint_every):
            w = replace(workload, vel=v0.detach().cpu().numpy().astype(np.float32),
                        wcsph=replace(workload.wcsph, viscosity_strenght=float(nu),
                                      stiffness=float(k)))
            model = W.build_model(w)
            ro = Rollout(model, int(steps), int(checkpoint_every))
            ro.forward()
            ctx.rollout = ro
            return torch.from_numpy(ro.final_positions_by_id()).to(v0.dtype)

        @staticmethod
        def backward(ctx, grad_out):
            g = ctx.rollout.backward(grad_out.detach().cpu().numpy())
            dv0 = torch.from_numpy(g["dv0"]).to(grad_out.dtype)
            dnu = torch.tensor(g["dnu"], dtype=grad_out.dtype)
            dk = torch.tensor(g["dk"], dtype=grad_out.dtype)
            return dv0, dnu, dk, None, None, None

    return WCSPHRollout
