"""MPM <-> rigid coupling with kinematic colliders.

The reference couples MPM with its rigid solver inside the grid op (legacy_coupler.py:389-403):
every grid node near a rigid geom has its velocity projected against the geom (friction,
restitution, SDF influence) and the momentum change is applied back to the rigid link.  Without a
rigid solver, a `Collider` is the geom: its pose and velocity are given by the caller every step
(a kinematic body, or the rigid solver of the host application), and the reaction force and
torque the particles exert on it are read back with `MPMSolver.get_collider_forces()`.

Coupling parameters default to gs.materials.Rigid's (materials/rigid.py:81-84).

A rigid geom whose SDF the reference samples on a voxel grid (boxes, meshes) is a collider of
shape "sdf" with an `SDFGrid` (values and gradients).  A tool entity (engine/entities/tool_entity:
a kinematic mesh with a voxel SDF, friction and softness, coupled before the rigid geoms) is a
collider of shape "tool" with an `SDFGrid` of values; the library moves it every substep from its
linear and angular velocity, as ToolEntity.advect does.  Grids come from the caller (the reference
builds them from meshes with trimesh/igl, which are not part of this library);
`SDFGrid.from_function` samples an analytic distance function.
"""

from __future__ import annotations

import dataclasses

import numpy as np

from . import _lib
from .exceptions import GenesisException

_TYPES = {"sphere": _lib.COLLIDER_SPHERE, "plane": _lib.COLLIDER_PLANE, "box": _lib.COLLIDER_BOX,
          "sdf": _lib.COLLIDER_SDF, "tool": _lib.COLLIDER_TOOL}


@dataclasses.dataclass(eq=False)
class SDFGrid:
    """Voxel signed-distance grid in the layout of the reference's SDF data (utils/sdf.py,
    tool_entity/mesh.py): values [r0, r1, r2] in mesh-frame distance units, gradients
    [r0, r1, r2, 3] (rigid geoms; None for a tool), T_mesh_to_sdf the 4x4 map from the mesh frame
    to voxel coordinates, cell_size the voxel edge in mesh units, sdf_max the largest value."""

    values: np.ndarray
    T_mesh_to_sdf: np.ndarray
    grads: np.ndarray | None = None
    cell_size: float = 1.0
    sdf_max: float = 0.0

    @classmethod
    def from_function(cls, sdf, lower, upper, res: int, grads: bool = True) -> "SDFGrid":
        """Sample `sdf` (callable on [n, 3] mesh-frame points) on a res^3 lattice spanning the box
        [lower, upper]; gradients by central differences of half a voxel."""
        lower = np.asarray(lower, np.float64)
        upper = np.asarray(upper, np.float64)
        cell = (upper - lower) / (res - 1)
        if not np.allclose(cell, cell[0]):
            raise GenesisException("SDFGrid.from_function needs a cube (equal voxel edges).")
        ax = [lower[d] + cell[d] * np.arange(res) for d in range(3)]
        pts = np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3)
        vals = np.asarray(sdf(pts), np.float64).reshape(res, res, res)
        g = None
        if grads:
            h = 0.5 * cell[0]
            g = np.stack([(np.asarray(sdf(pts + h * e)) - np.asarray(sdf(pts - h * e))) / (2 * h)
                          for e in np.eye(3)], -1).reshape(res, res, res, 3)
        T = np.eye(4)
        T[:3, :3] /= cell[0]
        T[:3, 3] = -lower / cell[0]
        return cls(values=vals.astype(np.float32), T_mesh_to_sdf=T,
                   grads=None if g is None else g.astype(np.float32), cell_size=float(cell[0]),
                   sdf_max=float(vals.max()))


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
    sdf: SDFGrid | None = None  # shapes "sdf" and "tool"
    floor_height: float = 0.0  # "tool": ToolOptions.floor_height

    def to_c(self, sdf_id: int = -1) -> "_lib.MpmCollider":
        if self.shape not in _TYPES:
            raise GenesisException(f"Unsupported collider shape: {self.shape}.")
        if self.shape in ("sdf", "tool") and (self.sdf is None or sdf_id < 0):
            raise GenesisException(f"A '{self.shape}' collider needs an SDFGrid.")
        if self.shape == "sdf" and self.sdf.grads is None:
            raise GenesisException("An 'sdf' collider needs an SDFGrid with gradients.")
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
        c.sdf_grid = int(sdf_id)
        c.floor_height = float(self.floor_height)
        return c


def tool(sdf: SDFGrid, pos=(0.0, 0.0, 0.0), quat=(1.0, 0.0, 0.0, 0.0), vel=(0.0, 0.0, 0.0), ang=(0.0, 0.0, 0.0),
         friction: float = 0.0, coup_softness: float = 0.01, floor_height: float = 0.0, env: int = -1) -> Collider:
    """A tool entity's collider with gs.materials.Tool defaults (materials/tool.py:29-32)."""
    return Collider(shape="tool", sdf=sdf, pos=pos, quat=quat, lin_vel=vel, ang_vel=ang, coup_friction=friction,
                    coup_softness=coup_softness, floor_height=floor_height, env=env)
