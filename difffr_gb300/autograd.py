"""torch.autograd.Function around a DiffDFSPH rollout.

``rollout(sim, init_params, steps)`` sets every body's initial velocity and angular
velocity from ``init_params`` (n_bodies x 6: v0, omega0), resets the simulation, runs
``steps`` steps and returns the final rigid states (n_bodies x 13: x, q (w,x,y,z), v,
omega) as a tensor that autograd differentiates with respect to ``init_params``.

The derivative is the reference's gradient chain (the per-step rigid Jacobian blocks of
the selected gradient mode, BoundaryModel_Akinci2012::perform_chain_rule; with the
gradient manager on, RigidBodyGradientManager's chain over body pairs, which couples the
bodies through the contact solver's blocks), applied in reverse over the recorded step
matrices. Two schedules:

* direct (``checkpoint_every=None``): the forward pass accumulates the pair Jacobians
  and records one 13x13 matrix per body and step; the backward pass is one reverse sweep.
* checkpointed (``checkpoint_every=k``): the forward pass runs without Jacobians and
  keeps a device snapshot every k steps; the backward pass recomputes each k-step segment
  from its snapshot with Jacobians on (bit-identical replay) and chains the adjoint
  through the segments, last to first. Memory: one snapshot per k steps in HBM.

This mirrors what the reference's optimisation scripts do with a torch.autograd.Function
around the simulator (experiments/rigid_body_trajectory_optimization/python/
gradient-based-optimize.py:170-251), with the forward-mode tangents replaced by the
equivalent reverse sweep.
"""
from __future__ import annotations

import numpy as np
import torch


class DiffDFSPHRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, init_params, sim, steps, checkpoint_every):
        p = init_params.detach().to("cpu", torch.float64).numpy().reshape(sim.n_bodies, 6)
        for b in range(sim.n_bodies):
            sim.set_rigid_init(b, p[b, :3], p[b, 3:])
        segments = []
        if checkpoint_every:
            sim.set_gradient_enabled(False)
            sim.reset()
            done = 0
            while done < steps:
                n = min(int(checkpoint_every), steps - done)
                segments.append((sim.checkpoint_save(), n))
                sim.step(n)
                done += n
        else:
            sim.set_gradient_enabled(True)
            sim.reset()
            sim.step(steps)
        out = np.stack([sim.rigid_state_vector(b) for b in range(sim.n_bodies)])
        ctx.sim = sim
        ctx.segments = segments
        ctx.dtype = init_params.dtype
        ctx.device = init_params.device
        return torch.as_tensor(out, dtype=init_params.dtype, device=init_params.device)

    @staticmethod
    def backward(ctx, grad_out):
        sim = ctx.sim
        lam = grad_out.detach().to("cpu", torch.float64).numpy().reshape(sim.n_bodies, 13)
        if ctx.segments:
            mgr = sim.uses_manager
            if mgr:  # the manager's v0 and omega0 columns have separate step maps
                lam = np.stack([lam, lam])
            sim.set_gradient_enabled(True)
            for slot, n in reversed(ctx.segments):
                sim.checkpoint_restore(slot)
                sim.reset_gradient()
                sim.step(n)
                lam = sim.adjoint_sweep(lam)
                sim.checkpoint_free(slot)
            ctx.segments = []
            g = np.concatenate([lam[0][:, 7:10], lam[1][:, 10:13]], axis=1) if mgr else lam[:, 7:13]
        else:
            g = sim.backward(lam)
        return torch.as_tensor(np.ascontiguousarray(g), dtype=ctx.dtype, device=ctx.device), None, None, None


def rollout(sim, init_params: torch.Tensor, steps: int, checkpoint_every: int | None = None) -> torch.Tensor:
    """Final rigid states (n_bodies x 13) after `steps` steps from initial velocities
    `init_params` (n_bodies x 6); differentiable with respect to `init_params`."""
    return DiffDFSPHRollout.apply(init_params, sim, int(steps), checkpoint_every)
