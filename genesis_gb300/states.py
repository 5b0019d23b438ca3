"""State containers (genesis/engine/states/solvers.py:150-207, entities.py:41-101)."""

from __future__ import annotations

import torch


class MPMSolverState:
    """Particle state of all scenes: pos/vel [B,N,3], C/F [B,N,3,3], Jp [B,N], active [B,N] bool."""

    def __init__(self, B: int, N: int, device, requires_grad: bool = False):
        kw = dict(dtype=torch.float32, device=device)
        self.pos = torch.zeros((B, N, 3), **kw)
        self.vel = torch.zeros((B, N, 3), **kw)
        self.C = torch.zeros((B, N, 3, 3), **kw)
        self.F = torch.zeros((B, N, 3, 3), **kw)
        self.Jp = torch.zeros((B, N), **kw)
        self.active = torch.zeros((B, N), dtype=torch.bool, device=device)
        if requires_grad:
            for t in (self.pos, self.vel, self.C, self.F, self.Jp):
                t.requires_grad_(True)

    def serializable(self):
        for k in ("pos", "vel", "C", "F", "Jp", "active"):
            setattr(self, k, getattr(self, k).detach())
        return self


class MPMEntityState(MPMSolverState):
    """Same fields for one entity's particle range; `active` is an int tensor as in the reference."""

    def __init__(self, entity, s_global: int, B: int, N: int, device):
        super().__init__(B, N, device)
        self.entity = entity
        self.s_global = s_global


class ToolEntityState:
    """genesis/engine/states/entities.py (ToolEntityState): pos [B, 3], quat [B, 4] (w, x, y, z),
    vel [B, 3], ang [B, 3] of one tool entity at the current frame."""

    def __init__(self, entity, s_global: int, B: int, device):
        kw = dict(dtype=torch.float32, device=device)
        self.entity = entity
        self.s_global = s_global
        self.pos = torch.zeros((B, 3), **kw)
        self.quat = torch.zeros((B, 4), **kw)
        self.vel = torch.zeros((B, 3), **kw)
        self.ang = torch.zeros((B, 3), **kw)

    def serializable(self):
        for k in ("pos", "quat", "vel", "ang"):
            setattr(self, k, getattr(self, k).detach())
        return self


class SimState:
    """genesis/engine/states/solvers.py:5-43 (only the MPM solver state here)."""

    def __init__(self, s_global: int, f_local: int, mpm_state: MPMSolverState | None):
        self.s_global = s_global
        self.f_local = f_local
        self.solvers_state = [mpm_state]

    def __getitem__(self, i):
        return self.solvers_state[i]

    def __len__(self):
        return len(self.solvers_state)
