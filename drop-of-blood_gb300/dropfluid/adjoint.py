"""Autograd-Function-style wrapper of the discrete adjoint (closed box, FP32 or
mixed precision).

    traj = DropTrajectory(sim, checkpoint_every=8)
    dye = traj.forward(32)                 # dob_tape_forward
    loss, g = l2_loss(dye, target)
    grads = traj.backward(g)               # dob_tape_backward -> d loss / d initial state
    d_imp = traj.drop_impulse_grad(scene, drop)      # hard-edged drop: impulse
    g = traj.drop_grads(scene, 0)                    # soft-edged drop: impulse and centre

The forward keeps a checkpoint of (velocity, dye, pressure) every
`checkpoint_every` steps on the device; the backward recomputes one segment
at a time, so device memory grows with the checkpoint count and the segment
length, not with the number of steps.
"""
from __future__ import annotations

import numpy as np

from . import abi


def l2_loss(dye, target):
    """L = sum (dye - target)^2 in float64 and dL/d dye as float32."""
    d = np.asarray(dye, np.float64) - np.asarray(target, np.float64)
    return float(np.sum(d * d)), (2.0 * d).astype(np.float32)


class DropTrajectory:
    """forward(nsteps) -> final dye; backward(dye_grad) -> gradients of the
    initial state ("u", "v", "w": MAC faces, "dye", "p")."""

    def __init__(self, sim, checkpoint_every: int = 8):
        self.sim = sim
        self.k = int(checkpoint_every)
        self.nsteps = 0

    def forward(self, nsteps: int):
        self.sim.tape_forward(int(nsteps), self.k)
        self.nsteps = int(nsteps)
        return self.sim.get_field(abi.FIELD_CONC)

    def backward(self, dye_grad):
        if self.nsteps == 0:
            raise RuntimeError("backward before forward")
        self.sim.tape_backward(dye_grad)
        return self.sim.gradients()

    def drop_grads(self, scene, drop) -> dict:
        """For a soft-edged drop (edge_cells > 0) injected into the
        trajectory's initial state, after backward: d loss / d s for its
        velocity scaled by s (at s = 1) and d loss / d centre (world units)."""
        d = scene.drops[drop] if isinstance(drop, int) else drop
        if not d.edge_cells > 0.0:
            raise ValueError("position gradients need a soft-edged drop (edge_cells > 0)")
        c = scene.config
        scale = c.dx / c.dt
        g_imp, g_pos = self.sim.sphere_soft_grad(d.center, d.radius, d.edge_cells * c.dx, 1.0,
                                                 (0.0, d.w_cells_per_step * scale, 0.0),
                                                 d.noise_cells_per_step * scale, d.seed)
        return {"impulse": g_imp, "position": g_pos}

    def drop_impulse_grad(self, scene, drop) -> float:
        """d loss / d s for the drop's injected face velocity s * vel (the
        noise term is not scaled), after backward."""
        dx = scene.config.dx
        dt = scene.config.dt
        vel = (0.0, drop.w_cells_per_step * dx / dt, 0.0)
        return self.sim.sphere_impulse(drop.center, drop.radius, vel)
