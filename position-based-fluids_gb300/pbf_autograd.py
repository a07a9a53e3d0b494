"""torch.autograd.Function over the C-ABI's differentiable rollout.

Forward: write (x0, v0), set the XSPH factor c and the gravity vector g, run
`substeps` substeps with pbf_rollout_forward and return the final positions
[N, 3] by original particle index.  Backward: pbf_rollout_backward, which
returns dL/dv0, dL/dc and dL/dg over the rollout's fixed neighbour structure.

The reference has no gradients; this wrapper exists so that the adjoint
kernels can be checked against finite differences and the FP64 adjoint with
torch's own machinery.  Tensors are CPU float32; the simulation owns the
device memory.
"""
from __future__ import annotations

import numpy as np
import torch

import pbf


class PbfRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v0: torch.Tensor, visc: torch.Tensor, gravity: torch.Tensor, sim: "pbf.Simulation",
                params, x0: np.ndarray, substeps: int, checkpoint_every: int):
        n = sim.n
        p = pbf.PbfParameters.from_buffer_copy(params)
        p.viscosityFactor = float(visc)
        g = gravity.detach().double().numpy()
        p.gravityVectorEnable = 1
        p.gravityX, p.gravityY, p.gravityZ = float(g[0]), float(g[1]), float(g[2])
        sim.set_params(p)
        vel = np.zeros((n, 4), np.float32)
        vel[:, :3] = v0.detach().float().numpy()
        sim.write_state(np.ascontiguousarray(x0, np.float32).reshape(n, 4), vel)
        sim.rollout_forward(substeps, checkpoint_every)
        ctx.sim = sim
        return torch.from_numpy(sim.positions_by_id()[:, :3].copy())

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        sim = ctx.sim
        gx = np.zeros((sim.n, 4), np.float32)
        gx[:, :3] = grad_out.detach().float().numpy()
        dv, dc, dg = sim.rollout_backward(gx)
        return (torch.from_numpy(dv[:, :3].copy()), torch.tensor(dc, dtype=torch.float32),
                torch.from_numpy(dg.copy()), None, None, None, None, None)


def rollout(v0, visc, gravity, sim, params, x0, substeps, checkpoint_every=10):
    return PbfRollout.apply(v0, visc, gravity, sim, params, x0, substeps, checkpoint_every)
