"""torch.autograd.Function over the discrete adjoint of fixed-step RKF78.

``integrate(ctx, y0, mass, h, n_steps, checkpoint_every)`` returns the final
state as a torch tensor; ``backward`` runs ``sol_adjoint_backward`` and returns
the gradients with respect to the initial state and the masses.  Tensors are
float64 on the CPU (the engine copies them to and from its own device
buffers through the C-ABI).
"""
from __future__ import annotations

import numpy as np
import torch


class RKF78Integrate(torch.autograd.Function):
    @staticmethod
    def forward(fctx, y0, mass, engine_ctx, h, n_steps, checkpoint_every):
        engine_ctx.set_masses(mass.detach().cpu().numpy().astype(np.float64))
        y = engine_ctx.adjoint_forward(y0.detach().cpu().numpy().astype(np.float64), h, n_steps, checkpoint_every)
        fctx.engine_ctx = engine_ctx
        return torch.from_numpy(y)

    @staticmethod
    def backward(fctx, grad_y):
        dy0, dm = fctx.engine_ctx.adjoint_backward(grad_y.detach().cpu().numpy().astype(np.float64))
        return torch.from_numpy(dy0), torch.from_numpy(dm), None, None, None, None


def integrate(engine_ctx, y0, mass, h, n_steps, checkpoint_every=100):
    return RKF78Integrate.apply(y0, mass, engine_ctx, h, n_steps, checkpoint_every)
