"""MPM <-> rigid coupling with kinematic colliders.

The reference couples MPM with its rigid solver inside the grid op (legacy_coupler.py:389-403):
every grid node near a rigid geom has its velocity projected against the geom (friction,
restitution, SDF influence) and the momentum change is applied back to the rigid link.  Without a
rigid solver, a `Collider` is the geom: its pose and velocity are given by the caller every step
(a kinematic body, or the rigid solver of the host application), and the reaction force and
torque the particles exert on it are read back with `MPMSolver.get_collider_forces()`.

Coupling parameters default to gs.materials.Rigid's (materials/rigid.py:81-84).
"""

from __future__ import annotations

import dataclasses

import numpy as np

from . import _lib
from .exceptions import GenesisException

_TYPES = {"sphere": _lib.COLLIDER_SPHERE, "plane": _lib.COLLIDER_PLANE, "box": _lib.COLLIDER_BOX}


@dataclasses.dataclass
class Collider:
    shape: str  # "sphere" (radius), "plane" (normal, in the collider frame), "box" (half extents)
    pos: tuple = (0.0, 0.0, 0.0)
    quat: tuple = (1.0, 0.0, 0.0, 0.0)  # (w, x, y, z)
    radius: float = 0.0
    normal: tuple = (0.0, 0.0, 1.0)
    half_extents: tuple = (0.0, 0.0, 0.0)
    lin_vel: tuple = (0.0, 0.0, 0.0)
    ang_vel: tuple = (0.0, 0.0, 0.0)
    com: tuple | None = None  # point the angular velocity turns about; defaults to pos
    coup_friction: float = 0.1
    coup_softness: float = 0.002
    coup_restitution: float = 0.0
    env: int = -1  # environment (scene) index, or -1 for every environment

    def to_c(self) -> "_lib.MpmCollider":
        if self.shape not in _TYPES:
            raise GenesisException(f"Unsupported collider shape: {self.shape}.")
        if not 0.0 <= self.coup_restitution <= 1.0 or self.coup_friction < 0 or self.coup_softness < 0:
            raise GenesisException("coup_friction and coup_softness must be >= 0 and coup_restitution in [0, 1].")
        c = _lib.MpmCollider()
        c.type = _TYPES[self.shape]
        c.scene = int(self.env)
        c.pos[:] = tuple(float(v) for v in self.pos)
        q = np.asarray(self.quat, dtype=np.float64)
        c.quat[:] = tuple(q)
        if self.shape == "sphere":
            c.size[:] = (float(self.radius), 0.0, 0.0)
        elif self.shape == "plane":
            c.size[:] = tuple(float(v) for v in self.normal)
        else:
            c.size[:] = tuple(float(v) for v in self.half_extents)
        c.com[:] = tuple(float(v) for v in (self.pos if self.com is None else self.com))
        c.lin_vel[:] = tuple(float(v) for v in self.lin_vel)
        c.ang_vel[:] = tuple(float(v) for v in self.ang_vel)
        c.friction = float(self.coup_friction)
        c.softness = float(self.coup_softness)
        c.restitution = float(self.coup_restitution)
        return c
