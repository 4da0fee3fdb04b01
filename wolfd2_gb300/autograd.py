"""torch.autograd view of the library's adjoint, for validation.

``KineticEnergy.apply(u0, v0, lid, solver, prm, nsteps, every, weight)``
returns J = 0.5 * weight * sum(u^2 + v^2) over the momentum unknowns after
``nsteps`` plain FP64 steps from (u0, v0) with the lid face profile ``lid``;
``J.backward()`` fills u0.grad, v0.grad, lid.grad from the discrete adjoint
(wolfd2gpu_adjoint, one call for the whole gradient).  Inputs are CPU float64
tensors in the driver layout ((mnx+1, mny+1), read as Fortran-ordered
arrays); the solver keeps its own initial pressure (the last loaded p).
"""
from __future__ import annotations

import numpy as np
import torch

NORTH, VAR_U = 4, 1


class KineticEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, v0, lid, solver, prm, nsteps, every, weight, p0=None):
        def arr(t):
            return np.asfortranarray(t.detach().cpu().numpy().astype(np.float64))

        u, v = arr(u0), arr(v0)
        p = arr(p0) if p0 is not None else np.zeros_like(u)
        solver.set_face_profile(1, 1, NORTH, VAR_U, lid.detach().cpu().numpy().astype(np.float64))
        solver.load_fields(u, v, p)
        J, gu, gv, _, gl, _ = solver.adjoint(prm, nsteps, every, weight, profile=(1, 1, NORTH, VAR_U),
                                              nprof=lid.numel())
        ctx.save_for_backward(torch.from_numpy(np.ascontiguousarray(gu)).view_as(u0),
                              torch.from_numpy(np.ascontiguousarray(gv)).view_as(v0),
                              torch.from_numpy(gl.copy()).view_as(lid))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        gu, gv, gl = ctx.saved_tensors
        return gJ * gu, gJ * gv, gJ * gl, None, None, None, None, None, None
