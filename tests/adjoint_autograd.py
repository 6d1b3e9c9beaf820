"""torch.autograd.Function around nekgpu_adjoint_gradient (test use only).

Forward builds a FP64 fused context on the GPU machine with the given permittivity,
runs nsteps from the initial state and returns J = sum jw |E|^2; backward
returns grad_J * dJ/deps from the library's discrete adjoint.
"""
from __future__ import annotations

import numpy as np
import torch

from nekcem_gb300 import MaxwellGPU


class BoxProblem:
    """Everything but eps: mesh, source, initial state, probe weights, steps."""

    def __init__(self, N, nel, lo, hi, bc, H0, E0, jw, nsteps, dt, t0=0.0, source=None, stride=0):
        self.N, self.nel, self.lo, self.hi, self.bc = N, nel, lo, hi, bc
        self.H0, self.E0, self.jw = H0, E0, jw
        self.nsteps, self.dt, self.t0, self.source, self.stride = nsteps, dt, t0, source, stride
        self.form = "fused64"       # form of the gradient's forward steps
        self.host_snapshots = None  # pinned host snapshots for the binomial schedule
        self.recompute_mixed = None  # fused FP64: segments recomputed in mixed stages
        self.last_ms = None

    def context(self, eps: np.ndarray, form: str = "fused64") -> MaxwellGPU:
        g = MaxwellGPU.from_box(self.N, self.nel, self.lo, self.hi, self.bc, form=form,
                                permittivity=np.ascontiguousarray(eps, dtype=np.float64))
        if self.source:
            g.set_source(**self.source)
        g.set_state(self.H0, self.E0)
        return g

    def objective(self, eps: np.ndarray) -> float:
        """J by a plain forward run (nekgpu_step) -- the finite-difference leg."""
        g = self.context(eps)
        g.run(self.nsteps, self.t0, self.dt)
        _, E = g.get_state()
        g.close()
        return float(np.sum(self.jw * (E * E)))

    def gradient(self, eps: np.ndarray):
        g = self.context(eps, self.form)
        J, dJ, fms, ams = g.adjoint_gradient(self.nsteps, self.t0, self.dt, self.jw, self.stride,
                                             host_snapshots=self.host_snapshots,
                                             recompute_mixed=self.recompute_mixed)
        g.close()
        self.last_ms = (fms, ams)
        return J, dJ


class FieldEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps: torch.Tensor, problem: BoxProblem):
        J, dJ = problem.gradient(eps.detach().cpu().numpy())
        ctx.save_for_backward(torch.from_numpy(dJ).to(eps.device))
        return eps.new_tensor(J)

    @staticmethod
    def backward(ctx, grad_out):
        (dJ,) = ctx.saved_tensors
        return grad_out * dJ, None
